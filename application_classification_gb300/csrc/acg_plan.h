// acg_plan.h -- the data-graph and plan objects behind the C ABI (internal).
//
// A plan matches one "pattern spec": a single pattern, or a disjoint union of
// several patterns matched together (acg_batch).  Every statistic of the
// algorithm is per pattern edge (column) or per pattern vertex, so the union is
// exact for each member, provided that each column keeps its own pattern's
// quirk coverage (qlim) and each pattern vertex its own pattern's iteration
// count (iters_p).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <tuple>
#include <utility>
#include <vector>

#include "acg.h"
#include "acg_bp.cuh"
#include "acg_device.cuh"
#include "acg_internal.h"
#include "acg_iter.cuh"

struct acg_data {
  int device = 0;
  int Dn = 0, De = 0, Kv = 0, Ke = 0;
  const double* node_feats = nullptr;  // caller's device memory
  const double* edge_feats = nullptr;
  acg::Csr dcsr;              // grouped by destination; other = source vertex
  acg::Csr scsr;              // grouped by source; other = destination vertex
  int* pos_in_dst = nullptr;  // [De] dst-CSR row of each src-CSR position
  int num_sms = acg::kNumSMs;
  // FP32 copies of the features for the mixed path, built on first use:
  // nodes [Dn][kv32], edges [De][ke32] in dst-CSR order (rows zero-padded
  // to a multiple of 4 features: 16-byte rows).
  float* nf32 = nullptr;
  float* ef32 = nullptr;
  int kv32 = 0, ke32 = 0;
  // warp work splits, shared by every plan on this graph: key = (0 dst / 1 src
  // CSR, parts, positions per step, ranges per part, chunk divisor, chunk cap)
  std::map<std::tuple<int, int, int, int, int, int>, acg::WarpWork> work;
  std::vector<acg::DevBuf> owned;
};

namespace acg {
// States of a match recorded for the adjoint, indexed by t (0 = after init,
// t = after iteration t): f = VF' - cR and r = VR' - cF ([Dn][Pp]), MU_raw as
// hi + lo ([Dn][Pn]) and the iteration's statistics ([glob_doubles]); null
// where state t is not recorded.
// Also, per state s, the edge maxima M of state s ([Dn][Pp]) and their first
// maximal dst-CSR positions (the edge phase of iteration s + 1), where a[s]
// is set; ppos: scratch for the hub chunks' positions.
struct StateRec {
  std::vector<void*> f, r, mh, ml, m;
  std::vector<int*> a;
  std::vector<double*> glob;
  int* ppos = nullptr;
  void resize(int n) {
    f.assign(n, nullptr);
    r.assign(n, nullptr);
    mh.assign(n, nullptr);
    ml.assign(n, nullptr);
    m.assign(n, nullptr);
    a.assign(n, nullptr);
    glob.assign(n, nullptr);
  }
  bool has(int t) const { return t >= 0 && t < (int)f.size() && mh[t] != nullptr; }
  bool has_am(int s) const { return s >= 0 && s < (int)a.size() && a[s] != nullptr; }
};
struct AdjWork;  // the adjoint's checkpoints and work buffers (acg_adjoint.cu)
}  // namespace acg

struct acg_plan {
  acg_data* data = nullptr;
  int prec = ACG_PREC_FP64;
  int Pn = 0, Pe = 0, Pp = 0, Pnp = 0, iters = 0;  // iters: the largest member's count
  const double* pv = nullptr;  // pattern features (device): [Pn][Kv], [Pe][Ke]
  const double* pe = nullptr;
  int* pat = nullptr;          // pattern incidence (device)
  int* iters_p = nullptr;      // [Pn] iteration count of each vertex's pattern
  long long* qlim_col = nullptr;  // [Pp] quirk coverage of each column
  double* S_final = nullptr;   // [Pn] column LSE of MU_raw at each vertex's last iteration
  bool is_union = false;       // several patterns (the output is scattered)
  bool fill_at_run = false;    // workspaces shared with other plans: refill per match
  acg::GroupShape gs{32, 1};   // group shape of the init kernel (group form)
  int init_blocks = 1, cv_blocks = 1, ce_blocks = 1;
  bool init_warp = false;      // init pass in warp form (small patterns)
  int qcov = 0, Pqc = 0;       // quirk-buffer columns holding -dE; their padded count
  // warp work over the destination-sorted CSR (edge phase, and the quirk maxima
  // over in-edges) and over the source-sorted CSR (static per-vertex reductions)
  acg::WarpShape ws{32, 1};    // edge phase and source-side pass (all Pp columns)
  acg::WarpShape qws{32, 1};   // destination-side quirk pass (Pqc columns)
  acg::WarpWork ew, sw;
  int edge_blocks = 1, src_blocks = 1, vert_blocks = 1;
  int maxdeg = 0;              // max over pattern vertices of in- plus out-degree
  uint32_t* vsched = nullptr;  // vertex phase, warp form: per-lane schedule [vterms][32]
  int vterms = 0;
  // work buffers (element type per precision)
  void* dE = nullptr;
  void* vf = nullptr;
  void* vr[2] = {nullptr, nullptr};
  void* dEmin = nullptr;
  void* B = nullptr;
  void* CV = nullptr;
  void* CVlo = nullptr;        // mixed precision: low part of CV
  void* Rq = nullptr;          // [Dn][Pqc] quirk maxima over out-edges
  void* Fq = nullptr;          // [Dn][Pqc] quirk maxima over in-edges
  void* M = nullptr;           // [Dn][Pp] edge-phase maxima
  void* part_iter = nullptr;
  void* part_src = nullptr;    // [sw.npartial][3 Pp + Pqc] chunk rows of the source-side pass
  double* bpart = nullptr;
  double* gv = nullptr;        // [3 Pn]
  double* ge = nullptr;        // [max(Pe, Pqc)]
  double* gi[2] = {nullptr, nullptr};  // [glob_doubles(Pn, Pe)]
  // the large buffers above as (bytes, field) in allocation order; a batch
  // allocates the largest of each over its plans once and binds them
  std::vector<std::pair<size_t, void**>> big;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int kernel_timing = 0;
  std::vector<cudaEvent_t> kev;  // [3 * iters] around each iteration's phases
  cudaStream_t last_stream = nullptr;
  int64_t launches = 0;
  bool ran = false;
  bool cdist_tc = false;       // edge cost matrix on the tensor cores
  bool edge_costs_ready = false;  // the next match finds dE already written (one-shot host call)
  void* dEq = nullptr;         // [De][dEq_cols]: the covered columns of dE, written with it
  int dEq_cols = 0;            // (0: none; the quirk pass then reads dE)
  bool cdist_tc_v = false;     // vertex cost matrix on the tensor cores
  bool edge_tc = false;        // edge phase recomputes the costs on the tensor cores:
  acg::WarpWork etw;           // its item split (one part per CTA),
  float* et_part = nullptr;    // partial rows of heavy-vertex chunks [npartial][Pp]
  int* et_hcnt = nullptr;      // and chunks done per heavy vertex
  int* heavy_ctr = nullptr;    // [nheavy] chunks of each heavy vertex done in this edge phase
  int* range_ctr = nullptr;    // [2] range claims and finished warps of the range-split
                               // kernels (one at a time on the plan's stream; each
                               // launch leaves both at zero)
  int* dev_err = nullptr;      // set by a device-side bounded wait that gave up
  double* cnull = nullptr;     // [Pe] C-null term, then [2 Pe] dE column stats (option cnull)
  double* cnull_part = nullptr;  // [3 Pe][cnull_blocks] block partials
  int* qmember = nullptr;        // [Pe] member of each union column (option cnull), else null
  int nmembers = 1;
  const acg::StateRec* rec = nullptr;  // states to record during a match (adjoint)
  acg::AdjWork* adj = nullptr;         // owned; freed by acg_plan_destroy
  std::vector<acg::DevBuf> owned;
};

namespace acg {

// What a plan matches, built on the host.
struct PatternSpec {
  int Pn = 0, Pe = 0;
  std::vector<int> pat;             // incidence, pattern_ints(Pn, Pe) layout
  std::vector<long long> qlim;      // [Pe] column q covers original edge ids < qlim[q]
  std::vector<int> iters_p;         // [Pn]
  const double* pv = nullptr;       // device [Pn][Kv]
  const double* pe = nullptr;       // device [Pe][Ke]
  bool is_union = false;
  std::vector<int> qmember;         // [Pe] member of each column (unions; empty: one member)
};

// Incidence arrays of a pattern from its endpoints (pattern_ints layout).
acg_status build_incidence(int pn, int pe, const uint64_t* ps, const uint64_t* pd,
                           std::vector<int>* pat);

// Validated options (defaults filled in).
acg_status resolve_options(const acg_options* opt, acg_options* o);

// Make a plan.  deferred: the large buffers are recorded in P->big, not
// allocated (the caller binds them; they are refilled on every match).
acg_status plan_create_impl(acg_data* D, PatternSpec&& spec, const acg_options& o,
                            cudaStream_t s, bool deferred, acg_plan** out);

// Scatter of a union's MU into its members' outputs: member i owns union
// vertices [p0[i], p0[i+1]) and writes out[i][v][p - p0[i]].
constexpr int kMaxUnion = 64;
struct UnionOut {
  int n = 0;
  double* out[kMaxUnion];
  int p0[kMaxUnion + 1];
};

// One whole match on stream s.  Single plans write mu_out [Dn][Pn]; union
// plans use mu_out as [Dn][Pn] scratch and scatter into uo.
acg_status run_match_any(acg_plan* P, double* mu_out, cudaStream_t s, const UnionOut* uo);

// Iteration t alone (edge phase, vertex phase, statistics), from the working
// state of iteration t - 1 (vf, vr[(t-1) & 1], gi[(t-1) & 1]); records state t
// when P->rec asks for it.  mu_out is written only on the last iteration.
acg_status run_iteration_any(acg_plan* P, int t, double* mu_out, cudaStream_t s);

// The C-null term of a plan with the cnull option (acg_cnull.cu), from its dE.
acg_status run_cnull(acg_plan* P, cudaStream_t s);
int cnull_blocks(int num_sms);

// Frees the adjoint's buffers of a plan (acg_adjoint.cu).
void adj_free(acg_plan* P);

}  // namespace acg
