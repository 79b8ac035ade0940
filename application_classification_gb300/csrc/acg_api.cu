// acg_api.cu -- the C ABI (include/acg.h): data graphs, plans, the match.
//
// A match runs, on the caller's stream:
//   cdist (vertex)  -> column stats  -> cdist (edge, dst-CSR order) -> stats
//   static source pass (dEmin, B, quirk maxima) + destination pass (quirk maxima)
//   init vertex pass (CV, MU0, first VF/VR)  -> stats
//   num_iters x { fused edge + vertex pass -> stats }
//   output: mu[v][p] -= S[p]
// which is main.cu:107-247 (prep, loop, transpose) of the reference.
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cstring>
#include <limits>
#include <memory>
#include <type_traits>
#include <vector>

#include "acg.h"
#include "acg_bp.cuh"
#include "acg_device.cuh"
#include "acg_internal.h"
#include "acg_cdist.cuh"
#include "acg_static.cuh"
#include "acg_iter.cuh"
#include "acg_plan.h"

using namespace acg;


namespace {
acg_status ensure_f32(acg_data* D, cudaStream_t s) {
  if (D->nf32) return ACG_OK;
  D->kv32 = (D->Kv + 3) / 4 * 4;
  D->ke32 = (D->Ke + 3) / 4 * 4;
  float *nf = nullptr, *ef = nullptr;
  ACG_TRY(dev_alloc(&D->owned, sizeof(float) * (size_t)D->Dn * std::max(1, D->kv32), (void**)&nf, s));
  ACG_TRY(dev_alloc(&D->owned, sizeof(float) * (size_t)D->De * std::max(1, D->ke32), (void**)&ef, s));
  ACG_TRY(launch_convert_rows(D->node_feats, nullptr, D->Dn, D->Kv, nf, D->kv32, s));
  ACG_TRY(launch_convert_rows(D->edge_feats, D->dcsr.eid, D->De, D->Ke, ef, D->ke32, s));
  D->nf32 = nf;
  D->ef32 = ef;
  return ACG_OK;
}

// cdist of the vertex and edge features, per precision.
template <typename T>
struct Cdist;
template <>
struct Cdist<double> {
  static acg_status run(acg_plan* P, acg_data* D, long long lim, cudaStream_t s);
};
template <>
struct Cdist<float> {
  static acg_status run(acg_plan* P, acg_data* D, long long lim, cudaStream_t s);
};
}  // namespace


namespace {

__global__ void validate_edges_kernel(const uint64_t* __restrict__ srcs,
                                      const uint64_t* __restrict__ dsts, long long m,
                                      unsigned long long n, uint32_t* __restrict__ s32,
                                      uint32_t* __restrict__ d32, int* __restrict__ bad) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const uint64_t s = srcs[i], d = dsts[i];
  if (s >= n || d >= n) {
    atomicOr(bad, 1);
    s32[i] = 0;
    d32[i] = 0;
    return;
  }
  s32[i] = (uint32_t)s;
  d32[i] = (uint32_t)d;
}

__global__ void invert_kernel(const int* __restrict__ eid, int m, int* __restrict__ inv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) inv[eid[i]] = i;
}

__global__ void compose_kernel(const int* __restrict__ seid, const int* __restrict__ inv, int m,
                               int* __restrict__ pos) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < m) pos[j] = inv[seid[j]];
}

__global__ void mu_from_cv_kernel(double* __restrict__ mu, const void* __restrict__ cv,
                                  const float* __restrict__ cvlo, int fp64,
                                  const double* __restrict__ gv, long long n, int Pn, int Pnp) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p = (int)(i % Pn);
  const long long ci = (i / Pn) * Pnp + p;
  const double c = fp64 ? ((const double*)cv)[ci]
                        : (double)((const float*)cv)[ci] + (double)cvlo[ci];
  // CV holds dV - LSE(dV); MU0 = -dV - LSE(-dV)
  mu[i] = -(c + gv[Pn + p]) - gv[2 * Pn + p];
}

// out[m][v][p - p0[m]] = mu[v][p] - S[p] for the member m owning union vertex p
__global__ void union_scatter_kernel(const double* __restrict__ mu, const double* __restrict__ S,
                                     long long n, int Pn, const UnionOut uo) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long v = i / Pn;
  const int p = (int)(i - v * Pn);
  int m = 0;
  while (m + 1 < uo.n && uo.p0[m + 1] <= p) ++m;
  const int w = uo.p0[m + 1] - uo.p0[m];
  uo.out[m][v * w + (p - uo.p0[m])] = mu[i] - S[p];
}

int elem_bytes(int prec) { return prec == ACG_PREC_FP64 ? 8 : 4; }

acg_status check_graph(const acg_graph* g, const char* what, bool need_feats) {
  if (!g) return set_error(ACG_ERR_INVALID_ARGUMENT, "%s graph is null", what);
  if (g->num_nodes > 0x7fffffffull || g->num_edges > 0x7fffffffull)
    return set_error(ACG_ERR_UNSUPPORTED, "%s graph: more than 2^31-1 vertices or edges",
                     what);
  if (need_feats) {
    if (g->num_nodes && g->node_feat_dim && !g->node_feats)
      return set_error(ACG_ERR_INVALID_ARGUMENT, "%s graph: node_feats is null", what);
    if (g->num_edges && g->edge_feat_dim && !g->edge_feats)
      return set_error(ACG_ERR_INVALID_ARGUMENT, "%s graph: edge_feats is null", what);
  }
  if (g->num_edges && (!g->srcs || !g->dsts))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "%s graph: srcs/dsts is null", what);
  return ACG_OK;
}

}  // namespace

namespace {

constexpr int kWorkOver = 3;  // per-item cost in load steps (item load, combine, store)

// Per vertex: its cost in load steps (0 without edges), summed into *total.
__global__ void work_cost_kernel(const int* __restrict__ off, int n, int step,
                                 unsigned long long* __restrict__ total) {
  __shared__ unsigned long long red[8];
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long c = 0;
  if (v < n) {
    const int deg = off[v + 1] - off[v];
    if (deg > 0) c = (unsigned long long)((deg + step - 1) / step + kWorkOver);
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(total, t);  // integer: the same in any order
  }
}

// Per vertex: its item count, partial-row count and hub flag for a chunk size.
__global__ void work_count_kernel(const int* __restrict__ off, int n, int chunk,
                                  uint32_t* __restrict__ nit, uint32_t* __restrict__ npart,
                                  uint32_t* __restrict__ hub) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const int deg = off[v + 1] - off[v];
  const uint32_t k = deg > chunk ? (uint32_t)((deg + chunk - 1) / chunk) : (deg > 0 ? 1u : 0u);
  nit[v] = k;
  npart[v] = deg > chunk ? k : 0u;
  hub[v] = deg > chunk ? 1u : 0u;
}

// Per vertex: its items (in order) with their costs, and its hub record.
__global__ void work_items_kernel(const int* __restrict__ off, int n, int chunk, int step,
                                  const uint32_t* __restrict__ ioff, const uint32_t* __restrict__ poff,
                                  const uint32_t* __restrict__ hoff, int4* __restrict__ items,
                                  unsigned long long* __restrict__ cost, int* __restrict__ hbase,
                                  int* __restrict__ hcount, int* __restrict__ hvert,
                                  int* __restrict__ pheavy) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= n) return;
  const int b = off[v], e = off[v + 1], deg = e - b;
  if (deg == 0) return;
  const uint32_t i0 = ioff[v];
  if (deg > chunk) {
    const int k = (deg + chunk - 1) / chunk;
    const int p0 = (int)poff[v], h = (int)hoff[v];
    hbase[h] = p0;
    hcount[h] = k;
    hvert[h] = v;
    for (int j = 0; j < k; ++j) {
      const int a = b + j * chunk, z = min(e, a + chunk);
      items[i0 + j] = make_int4(v, a, z, p0 + j);
      pheavy[p0 + j] = h;
      cost[i0 + j] = (unsigned long long)((z - a + step - 1) / step + kWorkOver);
    }
  } else {
    items[i0] = make_int4(v, b, e, -1);
    cost[i0] = (unsigned long long)((deg + step - 1) / step + kWorkOver);
  }
}

// split[w] (0 < w < nwarps) = 1 + the first item whose inclusive cost prefix
// reaches target * w (nitems if none), target = the items' total cost / nwarps;
// split[0] = 0, split[nwarps] = nitems.
__global__ void work_split_kernel(const unsigned long long* __restrict__ excl,
                                  const unsigned long long* __restrict__ cost, int nitems, int nwarps,
                                  int* __restrict__ split) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w > nwarps) return;
  if (w == 0) {
    split[0] = 0;
    return;
  }
  if (w == nwarps) {
    split[w] = nitems;
    return;
  }
  if (nitems == 0) {
    split[w] = 0;
    return;
  }
  const double target = ((double)excl[nitems - 1] + (double)cost[nitems - 1]) / nwarps;
  const double goal = target * w;
  int lo = 0, hi = nitems;  // first i with excl[i] + cost[i] >= goal
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((double)excl[mid] + (double)cost[mid] >= goal) hi = mid;
    else lo = mid + 1;
  }
  split[w] = lo < nitems ? lo + 1 : nitems;
}

}  // namespace

// The work split, built on the device: per-vertex costs and their total give
// the chunk size; per-vertex item counts, scanned, place the items (vertex
// order, chunks in order) and the hub records; a binary search of the 64-bit
// scanned item costs gives each part's boundary.  Items of a vertex are its
// in-edge positions (one item), or chunks of `chunk` positions for a heavy
// vertex; a part is a run of items of near-equal total cost.
acg_status acg::build_warp_work(const Csr& c, int nwarps, int step, WarpWork* out,
                                std::vector<DevBuf>* owned, cudaStream_t s, int max_ranges,
                                int chunk_div, int max_chunk) {
  const int n = c.n;
  if (nwarps < 1) return set_error(ACG_ERR_INVALID_ARGUMENT, "work split: %d warps", nwarps);
  if (n == 0) {  // no items: every part is empty
    WarpWork& W = *out;
    W = WarpWork{};
    W.nparts = nwarps;
    W.chunk = 4 * step;
    ACG_TRY(dev_alloc(owned, sizeof(int4), (void**)&W.items, s));
    ACG_TRY(dev_alloc(owned, sizeof(int) * ((size_t)nwarps + 1), (void**)&W.wsplit, s));
    ACG_TRY(dev_alloc(owned, sizeof(int), (void**)&W.hbase, s));
    ACG_TRY(dev_alloc(owned, sizeof(int), (void**)&W.hcount, s));
    ACG_TRY(dev_alloc(owned, sizeof(int), (void**)&W.hvert, s));
    ACG_TRY(dev_alloc(owned, sizeof(int), (void**)&W.pheavy, s));
    return ACG_OK;  // dev_alloc zero-fills: wsplit is all zeros
  }
  std::vector<DevBuf> tmp;
  struct TmpGuard {  // the temporaries go back on every exit path
    std::vector<DevBuf>* v;
    ~TmpGuard() { dev_free_all(v); }
  } guard{&tmp};
  auto fail = [&](acg_status st) {
    dev_free_all(&tmp);
    return st;
  };
  unsigned long long* total = nullptr;
  uint32_t *nit = nullptr, *npart = nullptr, *hub = nullptr;
  acg_status st = dev_alloc(&tmp, sizeof(unsigned long long) + 3 * sizeof(uint32_t), (void**)&total, s);
  if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(uint32_t) * ((size_t)n + 1), (void**)&nit, s);
  if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(uint32_t) * ((size_t)n + 1), (void**)&npart, s);
  if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(uint32_t) * ((size_t)n + 1), (void**)&hub, s);
  if (st != ACG_OK) return fail(st);
  work_cost_kernel<<<ceil_div(n, 256), 256, 0, s>>>(c.off, n, step, total);
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "work cost launch failed"));
  unsigned long long htotal = 0;
  ACG_CUDA_TRY(cudaMemcpyAsync(&htotal, total, sizeof(htotal), cudaMemcpyDeviceToHost, s));
  ACG_CUDA_TRY(cudaStreamSynchronize(s));
  const int nparts = work_parts((double)htotal, nwarps, max_ranges);
  const double per_part = (double)htotal / nparts;
  const long long cs = std::max(4LL, (long long)(per_part / chunk_div));  // chunk, in steps
  const int chunk = (int)std::min<long long>(std::max(1, max_chunk), cs * step);
  work_count_kernel<<<ceil_div(n, 256), 256, 0, s>>>(c.off, n, chunk, nit, npart, hub);
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "work count launch failed"));
  // counts -> offsets (the n-th entry, zero, becomes the total)
  ACG_TRY(scan_exclusive_u32(nit, nit, (size_t)n + 1, s));
  ACG_TRY(scan_exclusive_u32(npart, npart, (size_t)n + 1, s));
  ACG_TRY(scan_exclusive_u32(hub, hub, (size_t)n + 1, s));
  uint32_t tot[3] = {0, 0, 0};
  ACG_CUDA_TRY(cudaMemcpyAsync(&tot[0], nit + n, 4, cudaMemcpyDeviceToHost, s));
  ACG_CUDA_TRY(cudaMemcpyAsync(&tot[1], npart + n, 4, cudaMemcpyDeviceToHost, s));
  ACG_CUDA_TRY(cudaMemcpyAsync(&tot[2], hub + n, 4, cudaMemcpyDeviceToHost, s));
  ACG_CUDA_TRY(cudaStreamSynchronize(s));
  const int nitems = (int)tot[0], npartial = (int)tot[1], nheavy = (int)tot[2];
  WarpWork& W = *out;
  W = WarpWork{};
  W.nitems = nitems;
  W.nparts = nparts;
  W.chunk = chunk;
  W.nheavy = nheavy;
  W.npartial = npartial;
  ACG_TRY(dev_alloc(owned, sizeof(int4) * std::max(1, nitems), (void**)&W.items, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * ((size_t)nparts + 1), (void**)&W.wsplit, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * std::max(1, nheavy), (void**)&W.hbase, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * std::max(1, nheavy), (void**)&W.hcount, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * std::max(1, nheavy), (void**)&W.hvert, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * std::max(1, npartial), (void**)&W.pheavy, s));
  // per item (more items than vertices with hubs); the cost prefix in 64 bits
  // (a total can pass 2^32 on graphs with hundreds of millions of vertices)
  unsigned long long *cost = nullptr, *excl = nullptr;
  st = dev_alloc(&tmp, sizeof(unsigned long long) * ((size_t)nitems + 1), (void**)&cost, s);
  if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(unsigned long long) * ((size_t)nitems + 1), (void**)&excl, s);
  if (st != ACG_OK) return fail(st);
  work_items_kernel<<<ceil_div(n, 256), 256, 0, s>>>(c.off, n, chunk, step, nit, npart, hub, W.items, cost,
                                                     W.hbase, W.hcount, W.hvert, W.pheavy);
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "work items launch failed"));
  // exclusive prefix of the item costs; boundaries
  ACG_TRY(scan_exclusive_u64(cost, excl, (size_t)nitems, s));
  work_split_kernel<<<ceil_div(nparts + 1, 256), 256, 0, s>>>(excl, cost, nitems, nparts, W.wsplit);
  if (cudaGetLastError() != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "work split launch failed"));
  dev_free_on(&tmp, s);
  ACG_CUDA_TRY(cudaStreamSynchronize(s));
  return ACG_OK;
}

namespace {

template <typename T>
acg_status iterate(acg_plan* P, int t, double* mu_out, cudaStream_t s) {
  acg_data* D = P->data;
  const int Dn = D->Dn, Pn = P->Pn, Pe = P->Pe, Pp = P->Pp;
  if (P->kernel_timing) cudaEventRecord(P->kev[3 * (t - 1)], s);
  if constexpr (std::is_same_v<T, float>) {
    if (Pe > 0 && P->edge_tc && !P->rec) {  // costs recomputed on the tensor cores
      const WarpWork& w = P->etw;
      EdgeTcArgs ta{D->ef32, P->pe, D->dcsr.other, (const float*)P->vr[(t - 1) & 1], (float*)P->M,
                    w.items, w.wsplit, P->et_part, w.pheavy, w.hbase, w.hcount, w.hvert, P->et_hcnt,
                    P->dev_err, (long long)D->De, D->Ke, D->ke32, Pe, Pp};
      ACG_TRY(launch_edge_tc(ta, w.nparts, s));
      P->launches += 1;
      goto vertex_phase;
    }
  }
  if (Pe > 0) {
    EdgeMaxArgs<T> ea{P->ew.items, P->ew.nitems, P->ew.wsplit, D->dcsr.other,
                      (const T*)P->dE, (const T*)P->vr[(t - 1) & 1], (T*)P->M,
                      (T*)P->part_iter, Pp};
    ea.nranges = P->ew.nparts;
    ea.ctr = P->range_ctr;
    ea.pheavy = P->ew.pheavy;
    ea.hbase = P->ew.hbase;
    ea.hcount = P->ew.hcount;
    ea.hvert = P->ew.hvert;
    ea.hcnt = P->heavy_ctr;
    const bool am = P->rec && P->rec->has_am(t - 1);  // record M and its argmax of state t - 1
    if (am) {
      ea.argpos = P->rec->a[t - 1];
      ea.ppos = P->rec->ppos;
    }
    // FP32 without argmax: the hubs are combined inside the edge kernel
    const bool inside = sizeof(T) == 4 && !am;
    if (!inside) ea.hcnt = nullptr;
    ACG_TRY(launch_edge_max<T>(ea, P->ws, P->edge_blocks, s));
    if (am) {
      ACG_TRY(launch_heavy_combine_arg<T>((const T*)P->part_iter, P->rec->ppos, P->ew.hbase,
                                          P->ew.hcount, P->ew.hvert, P->ew.nheavy, Pp, (T*)P->M,
                                          P->rec->a[t - 1], s));
      ACG_CUDA_TRY(cudaMemcpyAsync(P->rec->m[t - 1], P->M, sizeof(T) * (size_t)Dn * Pp,
                                   cudaMemcpyDeviceToDevice, s));
    } else if (!inside) {
      ACG_TRY(launch_heavy_combine<T>((const T*)P->part_iter, P->ew.hbase, P->ew.hcount,
                                      P->ew.hvert, P->ew.nheavy, Pp, (T*)P->M, s));
    }
    P->launches += 1 + (!inside && P->ew.nheavy > 0);
  }
vertex_phase:
  if (P->kernel_timing) cudaEventRecord(P->kev[3 * (t - 1) + 1], s);
  VertexUpdArgs<T> va{D->dcsr.off, (const T*)P->M, (T*)P->vf, (T*)P->vr[t & 1],
                      (const T*)P->dEmin, (const T*)P->B, (const T*)P->CV,
                      (const T*)P->CVlo, P->gi[(t - 1) & 1], P->gi[t & 1], P->bpart,
                      mu_out, P->pat, Dn, Pn, Pe, Pp, P->Pnp, P->maxdeg, P->iters_p, t,
                      t == 1, t == P->iters};
  va.cnull = P->cnull;
  va.vsched = P->vsched;
  va.vterms = P->vterms;
  const bool rec = P->rec && P->rec->has(t);
  if (rec) {
    va.rec_f = (T*)P->rec->f[t];
    va.rec_r = (T*)P->rec->r[t];
    va.rec_mh = (T*)P->rec->mh[t];
    va.rec_ml = (T*)P->rec->ml[t];
  }
  ACG_TRY(launch_vertex_update<T>(va, P->vert_blocks, s));
  ACG_TRY(launch_finalize(P->bpart, P->vert_blocks,
                          StatSpec{2 * Pe, 2 * Pe + Pn, P->prec != ACG_PREC_FP64}, P->gi[t & 1], s));
  ACG_TRY(launch_capture_s(P->gi[t & 1] + 4 * Pe, P->iters_p, t, P->S_final, Pn, s));
  if (rec)
    ACG_CUDA_TRY(cudaMemcpyAsync(P->rec->glob[t], P->gi[t & 1], sizeof(double) * glob_doubles(Pn, Pe),
                                 cudaMemcpyDeviceToDevice, s));
  if (P->kernel_timing) cudaEventRecord(P->kev[3 * (t - 1) + 2], s);
  P->launches += 3;
  return ACG_OK;
}

// NVTX ranges over a match's phases, the phases the reference marks
// (main.cu:107-244): a tool attached to the process sees "acg_match" with the
// phase being enqueued nested in it; without a tool the calls cost next to
// nothing.
class MatchRanges {
 public:
  MatchRanges() { nvtxRangePushA("acg_match"); }
  ~MatchRanges() {
    if (inner_) nvtxRangePop();
    nvtxRangePop();
  }
  void phase(const char* name) {
    if (inner_) nvtxRangePop();
    nvtxRangePushA(name);
    inner_ = true;
  }

 private:
  bool inner_ = false;
};

template <typename T>
acg_status run_match(acg_plan* P, double* mu_out, cudaStream_t s, const UnionOut* uo) {
  MatchRanges ranges;
  acg_data* D = P->data;
  const int Dn = D->Dn, Pn = P->Pn, Pe = P->Pe, Pp = P->Pp;
  const long long De = D->De;
  const long long lim = (long long)Pn * (long long)Dn;
  P->launches = 0;
  cudaEventRecord(P->ev[0], s);
  if (P->fill_at_run) {  // shared workspaces: rows that no pass writes
    constexpr T inf = std::numeric_limits<T>::infinity();
    const size_t nv = (size_t)Dn * Pp, nq = (size_t)Dn * P->Pqc;
    ACG_TRY(launch_fill<T>((T*)P->M, nv, -inf, s));
    ACG_TRY(launch_fill<T>((T*)P->dEmin, nv, inf, s));
    ACG_TRY(launch_fill<T>((T*)P->B, nv, -inf, s));
    ACG_TRY(launch_fill<T>((T*)P->Rq, nq, -inf, s));
    ACG_TRY(launch_fill<T>((T*)P->Fq, nq, -inf, s));
    P->launches += 5;
  }
  ACG_CUDA_TRY(cudaMemsetAsync(P->S_final, 0, sizeof(double) * Pn, s));

  // ---- cdist (ac.hxx:33-56 via main.cu:109-110) + column stats
  ranges.phase("cost matrices");
  ACG_TRY(Cdist<T>::run(P, D, lim, s));
  ACG_TRY(run_cnull(P, s));
  cudaEventRecord(P->ev[1], s);
  // ---- static per-vertex reductions (acg_static.cu)
  ranges.phase("static passes");
  if (De > 0) {
    SrcStatsArgs<T> sa{P->sw.items, P->sw.nitems, P->sw.wsplit, D->pos_in_dst, D->scsr.eid,
                       (const T*)P->dE, (T*)P->dEmin, (T*)P->B, (T*)P->Rq,
                       (T*)P->part_src, P->qlim_col, De, lim, Pp, P->Pqc, P->qcov};
    sa.nranges = P->sw.nparts;
    sa.ctr = P->range_ctr;
    ACG_TRY(launch_src_stats<T>(sa, P->ws, P->src_blocks, s));
    ACG_TRY(launch_src_stats_combine<T>(sa, P->sw, s));
    DstQuirkArgs<T> qa{P->ew.items, P->ew.nitems, P->ew.wsplit, D->dcsr.eid,
                       (const T*)(P->dEq_cols ? P->dEq : P->dE),
                       (T*)P->Fq, (T*)P->part_iter, P->bpart, P->qlim_col, De, lim, Pp,
                       P->Pqc, P->qcov, P->ew.nparts};
    qa.dstride = P->dEq_cols;
    ACG_TRY(launch_dst_quirk<T>(qa, P->qws, P->edge_blocks, s));
    if (P->qcov > 0 && P->ew.nitems > 0) {  // ge[q < Pqc]; the later columns stay -inf
      ACG_TRY(launch_finalize(P->bpart, P->edge_blocks, StatSpec{0, P->Pqc}, P->ge, s));
      P->launches += 1;
    }
    if (P->qcov > 0)
      ACG_TRY(launch_heavy_combine<T>((const T*)P->part_iter, P->ew.hbase, P->ew.hcount,
                                      P->ew.hvert, P->ew.nheavy, P->Pqc, (T*)P->Fq, s));
    P->launches += 2 + (P->sw.nheavy > 0) + (P->qcov > 0 && P->ew.nheavy > 0);
  }
  // ---- init vertex pass
  ranges.phase("initial messages");
  {
    InitArgs<T> a{D->dcsr.off, D->scsr.off, (T*)P->CV, (T*)P->CVlo, (const T*)P->Rq,
                  (const T*)P->Fq, (const T*)P->B, (const T*)P->dEmin, (T*)P->vf,
                  (T*)P->vr[0], P->gv, P->ge, P->bpart, P->pat, De, lim, Dn, Pn, Pe, Pp,
                  P->Pnp, P->Pqc, P->qcov, P->qlim_col};
    const bool rec0 = P->rec && P->rec->has(0);
    if (rec0) {
      a.rec_f = (T*)P->rec->f[0];
      a.rec_mh = (T*)P->rec->mh[0];
      a.rec_ml = (T*)P->rec->ml[0];
    }
    if (P->init_warp)
      ACG_TRY(launch_init_warp<T>(a, P->init_blocks, s));
    else
      ACG_TRY(launch_init_vertex<T>(a, P->gs, P->init_blocks, s));
    // S = 0 (MU0 is normalised) and shifts 0 for the first pass
    ACG_CUDA_TRY(cudaMemsetAsync(P->gi[0] + 4 * Pe, 0,
                                 sizeof(double) * (glob_doubles(Pn, Pe) - 4 * Pe), s));
    ACG_TRY(launch_finalize(P->bpart, P->init_blocks, StatSpec{2 * Pe, 2 * Pe}, P->gi[0], s));
    P->launches += 2;
    if (rec0) {
      ACG_CUDA_TRY(cudaMemcpyAsync(P->rec->r[0], P->vr[0], sizeof(T) * (size_t)Dn * Pp,
                                   cudaMemcpyDeviceToDevice, s));
      ACG_CUDA_TRY(cudaMemcpyAsync(P->rec->glob[0], P->gi[0], sizeof(double) * glob_doubles(Pn, Pe),
                                   cudaMemcpyDeviceToDevice, s));
    }
  }
  cudaEventRecord(P->ev[2], s);
  // ---- BP iterations (main.cu:160-245): edge phase, heavy combine, vertex phase
  ranges.phase("iterations");
  for (int t = 1; t <= P->iters; ++t) ACG_TRY(iterate<T>(P, t, mu_out, s));
  ranges.phase("output");
  cudaEventRecord(P->ev[3], s);
  // ---- output [Dn][Pn] (main.cu:247 transpose is implicit in the layout)
  if (P->iters > 0 && !P->is_union) {
    ACG_TRY(launch_mu_output(mu_out, P->S_final, Dn, Pn, s));
  } else if (P->iters == 0) {
    const long long n = (long long)Dn * Pn;
    if (n > 0) {
      mu_from_cv_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(
          mu_out, P->CV, (const float*)P->CVlo, P->prec == ACG_PREC_FP64, P->gv, n, Pn, P->Pnp);
      ACG_LAUNCH_CHECK();
    }
  }
  if (P->is_union) {  // MU_raw - S_final into each member's output
    const long long n = (long long)Dn * Pn;
    if (n > 0 && uo) {
      union_scatter_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mu_out, P->S_final, n, Pn, *uo);
      ACG_LAUNCH_CHECK();
    }
  }
  P->launches += 1;
  cudaEventRecord(P->ev[4], s);
  return ACG_OK;
}

template <typename T, typename F>
acg_status run_cdist(acg_plan* P, acg_data* D, long long lim, const F* nf, int nfs, const F* ef,
                     int efs, bool gather, cudaStream_t s) {
  int vcols = P->cv_blocks;  // partial columns of the vertex statistics
  bool vdone = false;
  if constexpr (std::is_same_v<T, float> && std::is_same_v<F, float>) {
    if (P->cdist_tc_v) {
      ACG_TRY(launch_cdist_vertex_tc(nf, nfs, D->Kv, P->pv, P->Pn, P->Pnp, (float*)P->CV, P->bpart, D->Dn,
                                     P->cv_blocks, &vcols, P->dev_err, D->num_sms, s));
      vdone = true;
    }
  }
  if (!vdone) {
    CdistRbArgs<T, F> av{nf, nullptr, nullptr, P->pv, (T*)P->CV, P->bpart, D->Dn, D->De, lim,
                         D->Kv, nfs, P->Pn, P->Pnp, P->Pnp};
    ACG_TRY(launch_cdist_rb(av, kCdistVertex, P->cv_blocks, s));
  }
  ACG_TRY(launch_finalize(P->bpart, vcols, StatSpec{P->Pn, 2 * P->Pn}, P->gv, s));
  // rows in dst-CSR order; with no data edges the kernel writes empty partials
  CdistRbArgs<T, F> ae{ef, gather ? D->dcsr.eid : nullptr, D->dcsr.eid, P->pe, (T*)P->dE,
                       nullptr, D->De, D->De, lim, D->Ke, efs, P->Pe, P->Pp, P->Pp};
  if constexpr (std::is_same_v<T, float> && std::is_same_v<F, float>) {
    if (P->cdist_tc && P->edge_costs_ready) {  // written while the features were uploaded
      P->edge_costs_ready = false;
      P->launches += 2;
      return ACG_OK;
    }
    if (P->cdist_tc) {
      ACG_TRY(launch_cdist_edges_tc(ef, efs, D->Ke, P->pe, P->Pe, P->Pp, (float*)P->dE, D->De,
                                    P->dev_err, D->num_sms, s, nullptr,
                                    P->dEq_cols ? (float*)P->dEq : nullptr, P->dEq_cols));
      P->launches += 3;
      return ACG_OK;
    }
  }
  ACG_TRY(launch_cdist_edges(ae, P->ce_blocks, s));
  P->launches += 3;
  return ACG_OK;
}

acg_status Cdist<double>::run(acg_plan* P, acg_data* D, long long lim, cudaStream_t s) {
  return run_cdist<double, double>(P, D, lim, D->node_feats, D->Kv, D->edge_feats, D->Ke, true, s);
}

acg_status Cdist<float>::run(acg_plan* P, acg_data* D, long long lim, cudaStream_t s) {
  return run_cdist<float, float>(P, D, lim, D->nf32, D->kv32, D->ef32, D->ke32, false, s);
}

}  // namespace

// ------------------------------------------------------------ plan creation
namespace acg {

acg_status build_incidence(int pn, int pe, const uint64_t* ps, const uint64_t* pd,
                           std::vector<int>* out) {
  std::vector<int>& pat = *out;
  pat.assign(pattern_ints(pn, pe), 0);
  int* psrc = pat.data();
  int* pdst = psrc + pe;
  int* inoff = pdst + pe;
  int* inq = inoff + pn + 1;
  int* outoff = inq + pe;
  int* outq = outoff + pn + 1;
  for (int q = 0; q < pe; ++q) {
    if (ps[q] >= (uint64_t)pn || pd[q] >= (uint64_t)pn)
      return set_error(ACG_ERR_INDEX_OUT_OF_RANGE, "pattern edge %d endpoint >= %d", q, pn);
    psrc[q] = (int)ps[q];
    pdst[q] = (int)pd[q];
    inoff[pd[q] + 1]++;
    outoff[ps[q] + 1]++;
  }
  for (int p = 0; p < pn; ++p) {
    inoff[p + 1] += inoff[p];
    outoff[p + 1] += outoff[p];
  }
  std::vector<int> ci(inoff, inoff + pn), co(outoff, outoff + pn);
  for (int q = 0; q < pe; ++q) {  // ascending q within each vertex's lists
    inq[ci[pdst[q]]++] = q;
    outq[co[psrc[q]]++] = q;
  }
  return ACG_OK;
}

acg_status resolve_options(const acg_options* opt, acg_options* o) {
  acg_options_default(o);
  if (opt) *o = *opt;
  if (o->precision != ACG_PREC_FP64 && o->precision != ACG_PREC_MIXED)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "unknown precision %d", o->precision);
  if (o->cnull != 0 && o->cnull != 1)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "cnull must be 0 or 1 (got %d)", o->cnull);
  if (o->autotune != 0 && o->autotune != 1)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "autotune must be 0 or 1 (got %d)", o->autotune);
  if (o->cdist_kernel < 0 || o->cdist_kernel > 2)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "cdist_kernel must be 0, 1 or 2 (got %d)", o->cdist_kernel);
  if (o->edge_kernel < 0 || o->edge_kernel > 2)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "edge_kernel must be 0, 1 or 2 (got %d)", o->edge_kernel);
  return ACG_OK;
}

// At most kEdgeRanges item ranges per launched warp of the edge phase (fewer
// when a range would fall under kMinRangeSteps load steps): a warp does its
// own range, then claims others as it finishes.  Heavy-vertex chunks are as
// long as a range (chunk_div 1): with claimed ranges that leaves no tail, and
// fewer chunks mean fewer partial rows to write and combine.  RMAT-22 edge
// phase with fixed counts and quarter-range chunks: 1 range (a static split)
// 4.05 ms, 4: 3.76, 8: 3.49, 16: 3.41, 64: 3.53; 32 with range-long chunks
// 3.27 ms.  RMAT-18 wants fewer: 32 ranges of ~5 steps 0.27 ms, 16: 0.13.
#ifndef ACG_EDGE_RANGES
#define ACG_EDGE_RANGES 32
#endif
constexpr int kEdgeRanges = ACG_EDGE_RANGES;
#ifndef ACG_EDGE_CHUNK_DIV
#define ACG_EDGE_CHUNK_DIV 1
#endif
constexpr int kEdgeChunkDiv = ACG_EDGE_CHUNK_DIV;

// The work split for (CSR, parts, step, chunk divisor), built once per data graph.
static acg_status get_work(acg_data* D, int which, int nwarps, int step, WarpWork* out,
                           cudaStream_t s, int max_ranges = 1, int chunk_div = 4,
                           int max_chunk = 1 << 24) {
  const auto key = std::make_tuple(which, nwarps, step, max_ranges, chunk_div, max_chunk);
  auto it = D->work.find(key);
  if (it == D->work.end()) {
    WarpWork w;
    ACG_TRY(build_warp_work(which == 0 ? D->dcsr : D->scsr, nwarps, step, &w, &D->owned, s,
                            max_ranges, chunk_div, max_chunk));
    it = D->work.emplace(key, w).first;
  }
  *out = it->second;
  return ACG_OK;
}

acg_status plan_create_impl(acg_data* D, PatternSpec&& spec, const acg_options& o, cudaStream_t s,
                            bool deferred, acg_plan** out) {
  std::unique_ptr<acg_plan> P(new acg_plan());
  struct Guard {  // a plan that is not handed out frees what it holds on every exit path
    acg_plan* p;
    ~Guard() {
      if (!p) return;
      dev_free_all(&p->owned);
      for (auto& e : p->ev)
        if (e) cudaEventDestroy(e);
      for (auto& e : p->kev)
        if (e) cudaEventDestroy(e);
    }
  } guard{P.get()};
  P->data = D;
  P->prec = o.precision;
  P->Pn = spec.Pn;
  P->Pe = spec.Pe;
  P->iters = 0;
  for (int x : spec.iters_p) P->iters = std::max(P->iters, x);
  P->pv = spec.pv;
  P->pe = spec.pe;
  P->is_union = spec.is_union;
  P->fill_at_run = deferred;
  const int eb = elem_bytes(P->prec);
  const int W = 16 / eb;
  P->Pp = std::max(W, (P->Pe + W - 1) / W * W);
  P->Pnp = (P->Pn + W - 1) / W * W;
  const int Pn = P->Pn, Pe = P->Pe, Pp = P->Pp, Dn = D->Dn, De = D->De;
  auto fail = [&](acg_status st) {
    dev_free_all(&P->owned);
    return st;
  };
  acg_status st = ACG_OK;
  auto alloc = [&](size_t bytes, void** p) {
    if (st == ACG_OK) st = dev_alloc(&P->owned, bytes, p, s);
  };
  auto big = [&](size_t bytes, void** p) {  // the large workspaces
    if (deferred) {
      *p = nullptr;
      P->big.emplace_back(std::max<size_t>(bytes, 1), p);
    } else {
      alloc(bytes, p);
    }
  };
  alloc(sizeof(int) * spec.pat.size(), (void**)&P->pat);
  alloc(sizeof(int) * std::max(1, Pn), (void**)&P->iters_p);
  alloc(sizeof(long long) * Pp, (void**)&P->qlim_col);
  alloc(sizeof(double) * std::max(1, Pn), (void**)&P->S_final);
  alloc(sizeof(int), (void**)&P->dev_err);
  if (P->prec == ACG_PREC_MIXED && o.cdist_kernel != 1) {
    P->cdist_tc = cdist_tc_eligible(D->Ke, (D->Ke + 3) / 4 * 4, Pe, Pp);
    P->cdist_tc_v = cdist_tc_eligible(D->Kv, (D->Kv + 3) / 4 * 4, Pn, P->Pnp);
    if (o.cdist_kernel == 2 && !P->cdist_tc) {
      dev_free_all(&P->owned);
      return set_error(ACG_ERR_UNSUPPORTED,
                       "tensor-core cdist: edge feature dim %d, %d pattern edges", D->Ke, Pe);
    }
    if (o.cdist_kernel == 2 && !P->cdist_tc_v) {
      dev_free_all(&P->owned);
      return set_error(ACG_ERR_UNSUPPORTED,
                       "tensor-core cdist: vertex feature dim %d, %d pattern vertices", D->Kv, Pn);
    }
  }
  // the edge phase recomputing the costs (single plans with the tensor-core
  // edge cost matrix; a batch shares workspaces and keeps the stored matrix)
  if (P->prec == ACG_PREC_MIXED && o.edge_kernel == 2) {
    P->edge_tc = !deferred && P->cdist_tc && Pe > 0 && De > 0 &&
                 edge_tc_eligible(D->Ke, (D->Ke + 3) / 4 * 4, Pe, Pp);
    if (!P->edge_tc && o.edge_kernel == 2) {
      dev_free_all(&P->owned);
      return set_error(ACG_ERR_UNSUPPORTED,
                       "edge phase on the tensor cores: edge feature dim %d, %d pattern edges%s", D->Ke,
                       Pe, deferred ? " (batch)" : "");
    }
  }
  if (P->edge_tc) {
    st = get_work(D, 0, D->num_sms, 1, &P->etw, s, 1, 1, kEdgeTcChunk);
    alloc(sizeof(float) * (size_t)std::max(1, P->etw.npartial) * Pp, (void**)&P->et_part);
    alloc(sizeof(int) * (size_t)std::max(1, P->etw.nheavy), (void**)&P->et_hcnt);
  }
  if (o.cnull) {
    alloc(sizeof(double) * 3 * std::max(1, Pe), (void**)&P->cnull);
    alloc(sizeof(double) * 3 * std::max(1, Pe) * cnull_blocks(D->num_sms), (void**)&P->cnull_part);
    if (!spec.qmember.empty()) {  // a union: the normaliser runs per member
      alloc(sizeof(int) * spec.qmember.size(), (void**)&P->qmember);
      P->nmembers = 1 + *std::max_element(spec.qmember.begin(), spec.qmember.end());
    }
  }
  if (st != ACG_OK) return fail(st);
  std::vector<long long> qlim(Pp, 0);
  std::copy(spec.qlim.begin(), spec.qlim.end(), qlim.begin());
  ACG_CUDA_TRY(cudaMemcpyAsync(P->pat, spec.pat.data(), sizeof(int) * spec.pat.size(),
                               cudaMemcpyHostToDevice, s));
  if (P->qmember)
    ACG_CUDA_TRY(cudaMemcpyAsync(P->qmember, spec.qmember.data(), sizeof(int) * spec.qmember.size(),
                                 cudaMemcpyHostToDevice, s));
  if (Pn > 0)
    ACG_CUDA_TRY(cudaMemcpyAsync(P->iters_p, spec.iters_p.data(), sizeof(int) * Pn,
                                 cudaMemcpyHostToDevice, s));
  ACG_CUDA_TRY(cudaMemcpyAsync(P->qlim_col, qlim.data(), sizeof(long long) * Pp,
                               cudaMemcpyHostToDevice, s));
  // covered columns form a prefix (a union orders them first)
  P->qcov = 0;
  while (P->qcov < Pe && qlim[P->qcov] > 0) ++P->qcov;

  if (P->prec == ACG_PREC_MIXED) st = ensure_f32(D, s);
  if (st != ACG_OK) return fail(st);

  P->ws = choose_warp_shape(eb, Pp);
  // edge phase: one wave of resident blocks (8 warps each)
  {
    const int fit = eb == 8 ? edge_max_blocks_per_sm<double>(P->ws) : edge_max_blocks_per_sm<float>(P->ws);
    P->edge_blocks = D->num_sms * (o.edge_blocks_per_sm > 0 ? std::min(fit, o.edge_blocks_per_sm) : fit);
  }
  // item ranges for the launched warps: each warp's own, then claimed
  st = get_work(D, 0, P->edge_blocks * 8, edge_step(P->ws), &P->ew, s, kEdgeRanges, kEdgeChunkDiv);
  if (st != ACG_OK) return fail(st);
  st = dev_alloc(&P->owned, 2 * sizeof(int), (void**)&P->range_ctr, s);
  if (st == ACG_OK)
    st = dev_alloc(&P->owned, sizeof(int) * (size_t)std::max(1, P->ew.nheavy), (void**)&P->heavy_ctr, s);
  if (st != ACG_OK) return fail(st);
  // source-side static pass: one wave of resident blocks over the source CSR
  {
    const int fit = eb == 8 ? src_stats_blocks_per_sm<double>(P->ws) : src_stats_blocks_per_sm<float>(P->ws);
    P->src_blocks = D->num_sms * (o.edge_blocks_per_sm > 0 ? std::min(fit, o.edge_blocks_per_sm) : fit);
  }
  st = get_work(D, 1, P->src_blocks * 8, edge_step(P->ws), &P->sw, s, kEdgeRanges, kEdgeChunkDiv);
  if (st != ACG_OK) return fail(st);
  P->Pqc = std::max(W, (P->qcov + W - 1) / W * W);
  P->qws = choose_warp_shape(eb, P->Pqc);
  P->gs = choose_shape(eb, Pp, Pn);
  const int GPB = 256 / P->gs.G;
  const int nsm = D->num_sms;
  {
    const int* io = spec.pat.data() + 2 * Pe;  // in_off, then in_q, then out_off
    const int* oo = io + Pn + 1 + Pe;
    int md = 0;
    for (int p = 0; p < Pn; ++p) md = std::max(md, io[p + 1] - io[p] + oo[p + 1] - oo[p]);
    P->maxdeg = md;
    std::vector<uint32_t> vs;
    P->vterms = vertex_warp_schedule(spec.pat.data(), Pn, Pe, Pp, P->Pnp, &vs);
    if (P->vterms > 0) {
      st = dev_alloc(&P->owned, sizeof(uint32_t) * vs.size(), (void**)&P->vsched, s);
      if (st != ACG_OK) return fail(st);
      ACG_CUDA_TRY(cudaMemcpyAsync(P->vsched, vs.data(), sizeof(uint32_t) * vs.size(),
                                   cudaMemcpyHostToDevice, s));
    }
    P->vert_blocks = eb == 8 ? vertex_update_blocks<double>(Pn, Pe, Pp, P->Pnp, P->vterms, nsm, Dn)
                             : vertex_update_blocks<float>(Pn, Pe, Pp, P->Pnp, P->vterms, nsm, Dn);
    if (o.vertex_blocks_per_sm > 0)
      P->vert_blocks = std::min(P->vert_blocks, nsm * o.vertex_blocks_per_sm);
  }
  P->init_blocks = std::max(1, std::min(ceil_div(std::max(1, Dn), GPB), nsm * 4));
  {
    const int ib = eb == 8 ? init_warp_blocks<double>(Pn, Pe, Pp, nsm)
                           : init_warp_blocks<float>(Pn, Pe, Pp, nsm);
    if (ib > 0) {
      P->init_warp = true;
      P->init_blocks = ib;
    }
  }
  P->cv_blocks = std::max(1, std::min(ceil_div(std::max(1, Dn), 64), nsm * 2));
  // the tensor-core vertex matrix: up to four CTAs per SM (its per-tile chain
  // is latency-bound; the launch takes what fits, at most this many)
  if (P->cdist_tc_v) P->cv_blocks = std::max(1, std::min(ceil_div(std::max(1, Dn), 128), nsm * 4));
  P->ce_blocks = std::max(1, std::min(ceil_div(std::max(1, De), 256), nsm * 8));

  const size_t vrow = (size_t)Dn * Pp * eb;
  big((size_t)De * Pp * eb, &P->dE);
  // the covered columns (q < qcov, at most 16) also as compact rows, which the
  // quirk pass reads instead of whole cost rows; every plan has the slot (a
  // batch shares its plans' workspaces slot by slot)
  P->dEq_cols = (P->prec == ACG_PREC_MIXED && P->cdist_tc && P->qcov > 0 && P->Pqc <= 16) ? P->Pqc : 0;
  big(P->dEq_cols ? (size_t)De * P->dEq_cols * sizeof(float) : 1, &P->dEq);
  big(vrow, &P->vf);
  big(vrow, &P->vr[0]);
  big(vrow, &P->vr[1]);
  big(vrow, &P->dEmin);
  big(vrow, &P->B);
  big((size_t)Dn * P->Pqc * eb, &P->Rq);
  big((size_t)Dn * P->Pqc * eb, &P->Fq);
  big((size_t)Dn * P->Pnp * eb, &P->CV);
  if (P->prec == ACG_PREC_MIXED) big((size_t)Dn * P->Pnp * eb, &P->CVlo);
  big(vrow, &P->M);
  big((size_t)std::max(1, P->ew.npartial) * Pp * eb, &P->part_iter);
  big((size_t)std::max(1, P->sw.npartial) * (3 * Pp + P->Pqc) * eb, &P->part_src);
  if (!deferred && st == ACG_OK) {
    // rows that no pass writes: vertices without in-edges (M = -inf) or
    // without out-edges (dEmin = +inf, B = -inf, quirk maxima -inf)
    const size_t nv = (size_t)Dn * Pp, nq = (size_t)Dn * P->Pqc;
    if (eb == 8) {
      constexpr double inf = std::numeric_limits<double>::infinity();
      st = launch_fill<double>((double*)P->M, nv, -inf, s);
      if (st == ACG_OK) st = launch_fill<double>((double*)P->dEmin, nv, inf, s);
      if (st == ACG_OK) st = launch_fill<double>((double*)P->B, nv, -inf, s);
      if (st == ACG_OK) st = launch_fill<double>((double*)P->Rq, nq, -inf, s);
      if (st == ACG_OK) st = launch_fill<double>((double*)P->Fq, nq, -inf, s);
    } else {
      constexpr float inf = std::numeric_limits<float>::infinity();
      st = launch_fill<float>((float*)P->M, nv, -inf, s);
      if (st == ACG_OK) st = launch_fill<float>((float*)P->dEmin, nv, inf, s);
      if (st == ACG_OK) st = launch_fill<float>((float*)P->B, nv, -inf, s);
      if (st == ACG_OK) st = launch_fill<float>((float*)P->Rq, nq, -inf, s);
      if (st == ACG_OK) st = launch_fill<float>((float*)P->Fq, nq, -inf, s);
    }
  }
  const size_t bp = std::max({(size_t)(6 * Pe + 2 * Pn) * P->vert_blocks,
                              (size_t)5 * Pn * P->cv_blocks, (size_t)6 * Pe * P->init_blocks,
                              (size_t)2 * P->Pqc * P->edge_blocks});
  alloc(sizeof(double) * bp, (void**)&P->bpart);
  alloc(sizeof(double) * 3 * Pn, (void**)&P->gv);
  alloc(sizeof(double) * std::max(P->Pqc, Pe), (void**)&P->ge);
  if (st == ACG_OK)  // columns without covered elements (and the case De = 0)
    st = launch_fill<double>(P->ge, (size_t)std::max(P->Pqc, Pe), -std::numeric_limits<double>::infinity(), s);
  alloc(sizeof(double) * glob_doubles(Pn, Pe), (void**)&P->gi[0]);
  alloc(sizeof(double) * glob_doubles(Pn, Pe), (void**)&P->gi[1]);
  if (st != ACG_OK) return fail(st);
  for (auto& e : P->ev)
    if (cudaEventCreate(&e) != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "cudaEventCreate failed"));
  P->kernel_timing = o.kernel_timing;
  if (P->kernel_timing) {
    P->kev.assign(3 * (size_t)P->iters, nullptr);
    for (auto& e : P->kev)
      if (cudaEventCreate(&e) != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "cudaEventCreate failed"));
  }
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return fail(set_error(ACG_ERR_CUDA, "acg_plan_create: %s", cudaGetErrorString(cudaGetLastError())));
  guard.p = nullptr;
  *out = P.release();
  return ACG_OK;
}

acg_status run_iteration_any(acg_plan* P, int t, double* mu_out, cudaStream_t s) {
  return P->prec == ACG_PREC_FP64 ? iterate<double>(P, t, mu_out, s) : iterate<float>(P, t, mu_out, s);
}

acg_status run_match_any(acg_plan* P, double* mu_out, cudaStream_t s, const UnionOut* uo) {
  return P->prec == ACG_PREC_FP64 ? run_match<double>(P, mu_out, s, uo)
                                  : run_match<float>(P, mu_out, s, uo);
}

}  // namespace acg

namespace {

acg_status check_pattern(const acg_data* D, const acg_graph* pg) {
  if (pg->num_nodes == 0) return set_error(ACG_ERR_INVALID_ARGUMENT, "pattern has no vertices");
  if (pg->node_feat_dim != (uint64_t)D->Kv || pg->edge_feat_dim != (uint64_t)D->Ke)
    return set_error(ACG_ERR_INVALID_ARGUMENT,
                     "feature dims differ: data %d/%d, pattern %llu/%llu", D->Kv, D->Ke,
                     (unsigned long long)pg->node_feat_dim, (unsigned long long)pg->edge_feat_dim);
  if (pg->num_nodes > 128 || pg->num_edges > 256)
    return set_error(ACG_ERR_UNSUPPORTED,
                     "pattern with %llu vertices / %llu edges: at most 128 / 256 are supported",
                     (unsigned long long)pg->num_nodes, (unsigned long long)pg->num_edges);
  if (D->Kv > 1024 || D->Ke > 1024)
    return set_error(ACG_ERR_UNSUPPORTED, "feature dimension above 1024");
  return ACG_OK;
}

}  // namespace

extern "C" {

void acg_options_default(acg_options* opt) {
  if (!opt) return;
  std::memset(opt, 0, sizeof *opt);
  opt->precision = ACG_PREC_FP64;
  opt->num_iters = -1;
}

acg_status acg_data_create(const acg_graph* g, void* stream, acg_data** out) {
  clear_error();
  if (!out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_data_create: out is null");
  *out = nullptr;
  ACG_TRY(check_graph(g, "data", true));
  cudaStream_t s = (cudaStream_t)stream;
  std::unique_ptr<acg_data> D(new acg_data());
  ACG_CUDA_TRY(cudaGetDevice(&D->device));
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, D->device) == cudaSuccess && sms > 0)
    D->num_sms = sms;
  D->Dn = (int)g->num_nodes;
  D->De = (int)g->num_edges;
  D->Kv = (int)g->node_feat_dim;
  D->Ke = (int)g->edge_feat_dim;
  D->node_feats = g->node_feats;
  D->edge_feats = g->edge_feats;
  const int m = D->De, n = D->Dn;
  uint32_t *s32 = nullptr, *d32 = nullptr;
  int* bad = nullptr;
  std::vector<DevBuf> tmp;  // temporaries (zero-filled)
  auto fail = [&](acg_status st) {
    dev_free_all(&tmp);
    dev_free_all(&D->owned);
    return st;
  };
  {
    acg_status at = dev_alloc(&tmp, sizeof(uint32_t) * (size_t)(m ? m : 1), (void**)&s32, s);
    if (at == ACG_OK) at = dev_alloc(&tmp, sizeof(uint32_t) * (size_t)(m ? m : 1), (void**)&d32, s);
    if (at == ACG_OK) at = dev_alloc(&tmp, sizeof(int), (void**)&bad, s);
    if (at != ACG_OK) return fail(at);
  }
  if (m > 0) {
    validate_edges_kernel<<<ceil_div(m, 256), 256, 0, s>>>(g->srcs, g->dsts, m, (unsigned long long)n, s32, d32, bad);
    if (cudaGetLastError() != cudaSuccess) return fail(set_error(ACG_ERR_CUDA, "validate launch failed"));
  }
  int hbad = 0;
  if (cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return fail(set_error(ACG_ERR_CUDA, "acg_data_create: %s", cudaGetErrorString(cudaGetLastError())));
  if (hbad)
    return fail(set_error(ACG_ERR_INDEX_OUT_OF_RANGE,
                          "data graph: an edge endpoint is >= num_nodes (%d)", n));
  acg_status st = build_csr(d32, s32, n, m, &D->dcsr, &D->owned, s);
  if (st == ACG_OK) st = build_csr(s32, d32, n, m, &D->scsr, &D->owned, s);
  if (st == ACG_OK) st = dev_alloc(&D->owned, sizeof(int) * (size_t)m, (void**)&D->pos_in_dst, s);
  if (st == ACG_OK && m > 0) {
    int* inv = reinterpret_cast<int*>(s32);  // reuse: no longer needed
    invert_kernel<<<ceil_div(m, 256), 256, 0, s>>>(D->dcsr.eid, m, inv);
    compose_kernel<<<ceil_div(m, 256), 256, 0, s>>>(D->scsr.eid, inv, m, D->pos_in_dst);
    if (cudaGetLastError() != cudaSuccess) st = set_error(ACG_ERR_CUDA, "csr compose launch failed");
  }
  if (st == ACG_OK && cudaStreamSynchronize(s) != cudaSuccess)
    st = set_error(ACG_ERR_CUDA, "acg_data_create: %s", cudaGetErrorString(cudaGetLastError()));
  if (st != ACG_OK) return fail(st);
  dev_free_on(&tmp, s);
  *out = D.release();
  return ACG_OK;
}

acg_status acg_data_destroy(acg_data* D) {
  if (!D) return ACG_OK;
  dev_free_all(&D->owned);
  delete D;
  return ACG_OK;
}

acg_status acg_plan_create(acg_data* D, const acg_graph* pg, const acg_options* opt,
                           void* stream, acg_plan** out) {
  clear_error();
  if (!out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_plan_create: out is null");
  *out = nullptr;
  if (!D) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_plan_create: data is null");
  ACG_TRY(check_graph(pg, "pattern", true));
  acg_options o;
  ACG_TRY(resolve_options(opt, &o));
  ACG_TRY(check_pattern(D, pg));
  cudaStream_t s = (cudaStream_t)stream;
  const int Pn = (int)pg->num_nodes, Pe = (int)pg->num_edges;
  // pattern incidence (host build from the device endpoint arrays)
  std::vector<uint64_t> ps(Pe), pd(Pe);
  if (Pe > 0) {
    ACG_CUDA_TRY(cudaMemcpyAsync(ps.data(), pg->srcs, 8 * (size_t)Pe, cudaMemcpyDeviceToHost, s));
    ACG_CUDA_TRY(cudaMemcpyAsync(pd.data(), pg->dsts, 8 * (size_t)Pe, cudaMemcpyDeviceToHost, s));
    ACG_CUDA_TRY(cudaStreamSynchronize(s));
  }
  PatternSpec spec;
  spec.Pn = Pn;
  spec.Pe = Pe;
  ACG_TRY(build_incidence(Pn, Pe, ps.data(), pd.data(), &spec.pat));
  const long long lim = (long long)Pn * D->Dn;
  spec.qlim.resize(Pe);
  for (int q = 0; q < Pe; ++q) spec.qlim[q] = std::max(0LL, lim - (long long)q * D->De);
  spec.iters_p.assign(Pn, o.num_iters < 0 ? Pn : o.num_iters);
  spec.pv = pg->node_feats;
  spec.pe = pg->edge_feats;
  return plan_create_impl(D, std::move(spec), o, s, false, out);
}

acg_status acg_plan_destroy(acg_plan* P) {
  if (!P) return ACG_OK;
  adj_free(P);
  for (auto& e : P->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : P->kev)
    if (e) cudaEventDestroy(e);
  dev_free_all(&P->owned);
  delete P;
  return ACG_OK;
}

acg_status acg_match(acg_plan* P, double* mu_out, void* stream) {
  clear_error();
  if (!P) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_match: plan is null");
  if (!mu_out && (long long)P->data->Dn * P->Pn > 0)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_match: mu_out is null");
  cudaStream_t s = (cudaStream_t)stream;
  P->last_stream = s;
  if (P->data->Dn == 0) return ACG_OK;
  acg_status st = run_match_any(P, mu_out, s, nullptr);
  P->ran = st == ACG_OK;
  return st;
}

acg_status acg_plan_stats(acg_plan* P, acg_stats* out) {
  clear_error();
  if (!P || !out) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_plan_stats: null argument");
  std::memset(out, 0, sizeof *out);
  if (!P->ran) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_plan_stats: no match has run");
  ACG_CUDA_TRY(cudaEventSynchronize(P->ev[4]));
  {
    int err = 0;
    ACG_CUDA_TRY(cudaMemcpy(&err, P->dev_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err)
      return set_error(ACG_ERR_DEVICE_TIMEOUT,
                       "acg_plan_stats: a device-side wait of the last match gave up");
  }
  float t01 = 0, t12 = 0, t23 = 0, t04 = 0;
  cudaEventElapsedTime(&t01, P->ev[0], P->ev[1]);
  cudaEventElapsedTime(&t12, P->ev[1], P->ev[2]);
  cudaEventElapsedTime(&t23, P->ev[2], P->ev[3]);
  cudaEventElapsedTime(&t04, P->ev[0], P->ev[4]);
  out->ms_cdist = t01;
  out->ms_init = t12;
  out->ms_iters = t23;
  out->ms_total = t04;
  const double eb = elem_bytes(P->prec);
  const double Dn = P->data->Dn, De = P->data->De, Pe = P->Pe, Pn = P->Pn;
  // Algorithmic bytes (unpadded Pe).  Edge phase: per in-edge its dE row and
  // source index; each source's Z row read once; each M row written once; the
  // work items.  Vertex phase: M, Y, dEmin, B and CV (with its low part in
  // mixed precision) read, Y and Z written, the in-degree offsets.
  const double cvb = P->prec == ACG_PREC_MIXED ? 2.0 * eb : eb;
  out->bytes_edge_phase = De * (Pe * eb + 4.0) + 2.0 * Dn * Pe * eb + (double)P->ew.nitems * 16.0;
  if (P->edge_tc)  // costs recomputed: per in-edge its FP32 features and source
    out->bytes_edge_phase = De * (P->data->Ke * 4.0 + 4.0) + 2.0 * Dn * Pe * eb +
                            (double)P->etw.nitems * 16.0;
  out->bytes_vertex_phase = Dn * (4.0 * Pe * eb + Pn * cvb + 2.0 * Pe * eb + 4.0);
  out->bytes_iters = (out->bytes_edge_phase + out->bytes_vertex_phase) * P->iters;
  out->launches = P->launches;
  out->num_iters = P->iters;
  out->edge_warps = (int64_t)P->edge_blocks * 8;
  out->edge_ranges = P->ew.nparts;
  out->edge_heavy_vertices = P->ew.nheavy;
  if (P->kernel_timing) {
    double se = 0, sv = 0;
    for (int t = 0; t < P->iters; ++t) {
      float a = 0, b = 0;
      cudaEventElapsedTime(&a, P->kev[3 * t], P->kev[3 * t + 1]);
      cudaEventElapsedTime(&b, P->kev[3 * t + 1], P->kev[3 * t + 2]);
      se += a;
      sv += b;
    }
    out->ms_edge_phase = se;
    out->ms_vertex_phase = sv;
  }
  return ACG_OK;
}

acg_status acg_match_graphs(const acg_graph* data, const acg_graph* pattern,
                            const acg_options* opt, double* mu_out, void* stream) {
  acg_data* D = nullptr;
  ACG_TRY(acg_data_create(data, stream, &D));
  acg_plan* P = nullptr;
  acg_status st = acg_plan_create(D, pattern, opt, stream, &P);
  if (st == ACG_OK) st = acg_match(P, mu_out, stream);
  if (st == ACG_OK && cudaStreamSynchronize((cudaStream_t)stream) != cudaSuccess)
    st = set_error(ACG_ERR_CUDA, "acg_match_graphs: %s", cudaGetErrorString(cudaGetLastError()));
  acg_plan_destroy(P);
  acg_data_destroy(D);
  return st;
}

acg_status acg_release_cached_memory(void) {
  clear_error();
  cudaDeviceSynchronize();
  release_pools();
  return ACG_OK;
}

acg_status acg_inject_alloc_failure(int64_t nth) {
  clear_error();
  set_alloc_failure((long long)nth);
  return ACG_OK;
}

acg_status acg_device_memory_in_use(int64_t* bytes) {
  clear_error();
  if (!bytes) return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_device_memory_in_use: null argument");
  ACG_CUDA_TRY(cudaDeviceSynchronize());  // stream-ordered frees have happened
  const long long b = device_memory_in_use();
  if (b < 0) return set_error(ACG_ERR_CUDA, "acg_device_memory_in_use: no device");
  *bytes = (int64_t)b;
  return ACG_OK;
}

acg_status acg_match_graphs_host(const acg_graph* data, const acg_graph* pattern,
                                 const acg_options* opt, double* mu_out_host, void* stream) {
  clear_error();
  ACG_TRY(check_graph(data, "data", true));
  ACG_TRY(check_graph(pattern, "pattern", true));
  if (!mu_out_host && data->num_nodes * pattern->num_nodes > 0)
    return set_error(ACG_ERR_INVALID_ARGUMENT, "acg_match_graphs_host: mu_out_host is null");
  cudaStream_t s = (cudaStream_t)stream;
  cudaStream_t s2 = nullptr, s3 = nullptr;
  constexpr int kChunks = 16;  // edge-feature upload pieces (mixed precision)
  cudaEvent_t ev = nullptr, ev_nodes = nullptr, ev_csr = nullptr, ev_plan = nullptr, ev_chunk[kChunks] = {};
  std::vector<DevBuf> tmp;
  acg_data* D = nullptr;
  acg_plan* P = nullptr;
  acg_status st = ACG_OK;
  auto cuda_ok = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && st == ACG_OK)
      st = set_error(ACG_ERR_CUDA, "acg_match_graphs_host: %s: %s", what, cudaGetErrorString(e));
    return st == ACG_OK;
  };
  cuda_ok(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking), "stream");
  cuda_ok(cudaStreamCreateWithFlags(&s3, cudaStreamNonBlocking), "stream");
  for (cudaEvent_t* e : {&ev, &ev_nodes, &ev_csr, &ev_plan}) cuda_ok(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "event");
  for (auto& e : ev_chunk) cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  // Device copies of the four arrays of each graph: the endpoints (the CSRs
  // need them) and the pattern on `stream`, the data features on the second
  // stream while the CSRs are built.  The host link (~210 GB/s, the same for
  // copy engines and for kernels reading pinned memory) is the critical path,
  // so with mixed precision the edge features go up in pieces and a third
  // stream turns each piece, as it lands, into its FP32 rows (destination-CSR
  // order, through the inverse of the CSR's edge order) and, once the plan
  // exists, into its rows of the edge cost matrix: the match then starts with
  // dE written.  FP64 plans read the caller's FP64 features and wait for them.
  acg_graph dg = *data, pg = *pattern;
  const size_t m = data->num_edges, n = data->num_nodes;
  const bool mixed = opt && opt->precision == ACG_PREC_MIXED;
  const bool chunked = mixed && m > 0 && data->edge_feat_dim > 0 && n > 0 && data->node_feat_dim > 0;
  struct Up {
    const void* h;
    size_t bytes;
    int lane;  // 0: stream, 1: second stream, 2: second stream in pieces
    const void** out;
  };
  const Up ups[] = {
      {data->srcs, 8 * m, 0, (const void**)&dg.srcs},
      {data->dsts, 8 * m, 0, (const void**)&dg.dsts},
      {pattern->srcs, 8 * pattern->num_edges, 0, (const void**)&pg.srcs},
      {pattern->dsts, 8 * pattern->num_edges, 0, (const void**)&pg.dsts},
      {pattern->node_feats, 8 * pattern->num_nodes * pattern->node_feat_dim, 0, (const void**)&pg.node_feats},
      {pattern->edge_feats, 8 * pattern->num_edges * pattern->edge_feat_dim, 0, (const void**)&pg.edge_feats},
      {data->node_feats, 8 * n * data->node_feat_dim, 1, (const void**)&dg.node_feats},
      {data->edge_feats, 8 * m * data->edge_feat_dim, chunked ? 2 : 1, (const void**)&dg.edge_feats}};
  void* dptr[8] = {};
  for (int i = 0; i < 8 && st == ACG_OK; ++i)
    if (ups[i].h && ups[i].bytes) st = dev_alloc(&tmp, ups[i].bytes, &dptr[i], s);
  cuda_ok(cudaStreamSynchronize(s), "alloc");  // the allocations exist for every stream
  const size_t ke = data->edge_feat_dim;
  auto piece = [&](int c) { return std::make_pair(m * c / kChunks, m * (c + 1) / kChunks); };
  for (int i = 0; i < 8 && st == ACG_OK; ++i) {
    if (!dptr[i]) continue;
    if (ups[i].lane == 2) {
      for (int c = 0; c < kChunks && st == ACG_OK; ++c) {
        const auto [e0, e1] = piece(c);
        if (e1 > e0)
          cuda_ok(cudaMemcpyAsync((double*)dptr[i] + e0 * ke, (const double*)ups[i].h + e0 * ke,
                                  (e1 - e0) * ke * 8, cudaMemcpyHostToDevice, s2), "copy");
        cuda_ok(cudaEventRecord(ev_chunk[c], s2), "event record");
      }
    } else {
      cuda_ok(cudaMemcpyAsync(dptr[i], ups[i].h, ups[i].bytes, cudaMemcpyHostToDevice, ups[i].lane ? s2 : s),
              "copy");
    }
    if (st == ACG_OK) *ups[i].out = dptr[i];
    if (i == 6) cuda_ok(cudaEventRecord(ev_nodes, s2), "event record");
  }
  cuda_ok(cudaEventRecord(ev, s2), "event record");
  double* mu = nullptr;
  if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(double) * n * pattern->num_nodes, (void**)&mu, s);
  if (st == ACG_OK) st = acg_data_create(&dg, s, &D);  // reads the endpoints only
  int* pos = nullptr;
  float* x32 = nullptr;
  if (st == ACG_OK && chunked) {
    // the FP32 copies ensure_f32 would make, made here piece by piece
    D->kv32 = (D->Kv + 3) / 4 * 4;
    D->ke32 = (D->Ke + 3) / 4 * 4;
    float *nf = nullptr, *ef = nullptr;
    st = dev_alloc(&D->owned, sizeof(float) * (size_t)D->Dn * D->kv32, (void**)&nf, s);
    if (st == ACG_OK) st = dev_alloc(&D->owned, sizeof(float) * (size_t)D->De * D->ke32, (void**)&ef, s);
    if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(int) * (size_t)D->De, (void**)&pos, s);
    if (st == ACG_OK) st = dev_alloc(&tmp, sizeof(float) * (size_t)D->De * D->ke32, (void**)&x32, s);
    if (st == ACG_OK && cuda_ok(cudaEventRecord(ev_csr, s), "event record") &&
        cuda_ok(cudaStreamWaitEvent(s3, ev_csr, 0), "wait")) {
      st = launch_inverse_perm(D->dcsr.eid, D->De, pos, s3);
      if (st == ACG_OK && cuda_ok(cudaStreamWaitEvent(s3, ev_nodes, 0), "wait"))
        st = launch_convert_rows(D->node_feats, nullptr, D->Dn, D->Kv, nf, D->kv32, s3);
      D->nf32 = nf;  // the plan finds the copies made (on s3, which `stream` waits for below)
      D->ef32 = ef;
    }
  } else if (st == ACG_OK && mixed) {
    if (cuda_ok(cudaEventRecord(ev_csr, s), "event record") && cuda_ok(cudaStreamWaitEvent(s2, ev_csr, 0), "wait"))
      st = ensure_f32(D, s2);
    cuda_ok(cudaEventRecord(ev, s2), "event record");
  }
  if (st == ACG_OK && !mixed) cuda_ok(cudaStreamWaitEvent(s, ev, 0), "wait");
  if (st == ACG_OK) st = acg_plan_create(D, &pg, opt, s, &P);
  if (st == ACG_OK && chunked) {
    // each piece as it lands: FP32 rows, then (tensor-core plans) its rows of dE
    const bool costs = P->cdist_tc && P->Pe > 0;
    if (costs && cuda_ok(cudaEventRecord(ev_plan, s), "event record"))
      cuda_ok(cudaStreamWaitEvent(s3, ev_plan, 0), "wait");
    for (int c = 0; c < kChunks && st == ACG_OK; ++c) {
      const auto [e0, e1] = piece(c);
      if (e1 <= e0 || !cuda_ok(cudaStreamWaitEvent(s3, ev_chunk[c], 0), "wait")) continue;
      st = launch_convert_scatter(D->edge_feats, (long long)e0, (long long)e1, D->Ke, pos, x32, D->ef32,
                                  D->ke32, s3);
      if (st == ACG_OK && costs)
        st = launch_cdist_edges_tc(x32 + e0 * D->ke32, D->ke32, D->Ke, P->pe, P->Pe, P->Pp, (float*)P->dE,
                                   (long long)(e1 - e0), P->dev_err, D->num_sms, s3, pos + e0,
                                   P->dEq_cols ? (float*)P->dEq : nullptr, P->dEq_cols);
    }
    if (st == ACG_OK) P->edge_costs_ready = costs;
    cuda_ok(cudaEventRecord(ev, s3), "event record");
  }
  if (st == ACG_OK && mixed) cuda_ok(cudaStreamWaitEvent(s, ev, 0), "wait");
  if (st == ACG_OK) st = acg_match(P, mu, s);
  if (st == ACG_OK && n * pattern->num_nodes > 0)
    cuda_ok(cudaMemcpyAsync(mu_out_host, mu, sizeof(double) * n * pattern->num_nodes,
                            cudaMemcpyDeviceToHost, s), "copy back");
  if (st == ACG_OK) cuda_ok(cudaStreamSynchronize(s), "synchronise");
  if (s2) cudaStreamSynchronize(s2);
  if (s3) cudaStreamSynchronize(s3);
  acg_plan_destroy(P);
  acg_data_destroy(D);
  dev_free_all(&tmp);
  for (cudaEvent_t e : {ev, ev_nodes, ev_csr, ev_plan})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ev_chunk)
    if (e) cudaEventDestroy(e);
  if (s2) cudaStreamDestroy(s2);
  if (s3) cudaStreamDestroy(s3);
  return st;
}

}  // extern "C"
