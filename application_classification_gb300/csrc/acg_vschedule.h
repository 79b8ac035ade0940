// acg_vschedule.h -- the vertex phase's per-lane schedule of its compensated
// MU_raw sums (warp form of vertex_warp_kernel, acg_iter.cu), host code that
// nvcc and the host compiler both build (the CPU tests compile it directly).
//
// A warp stages kVps data vertices at a time.  Each (staged vertex jv, pattern
// vertex p) sum is one job: the terms -CV[jv][p], then F[jv][q] for the in-edges
// q of p (dst_q = p) ascending, then R[jv][q] for its out-edges (src_q = p)
// ascending -- the order of the tile form.  The jobs go to the 32 lanes longest
// first, each to the least loaded lane, so a lane runs ~1/32 of the stage's terms
// instead of the largest pattern degree for every vertex.  Every sum keeps its
// terms and their order, so the result does not depend on the spread.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#ifdef __CUDACC__
#define ACG_VS_HD __host__ __device__
#else
#define ACG_VS_HD
#endif

namespace acg {

// schedule word: element offset of the term in the stage (bits 0-11), first
// term of its job (bit 12), last term (bit 13), the job's slot
// jv * (32 PPL + 1) + p in the per-warp MU_raw rows (bits 16-24); stored
// [t / 4][lane][t % 4] so that a lane's four next words are one 16-byte load
constexpr uint32_t kSchedStart = 1u << 12, kSchedEnd = 1u << 13;

// Element offsets of one stage of vps vertices: M, Y, dEmin, B rows [vps][Pp],
// then the CV rows [vps][Pnp] and (FP32) their low parts.
struct VwStage {
  int oM, oY, oE, oB, oC, oCl, n;
  ACG_VS_HD VwStage(int Pp, int Pnp, bool lo, int vps) {
    oM = 0;
    oY = vps * Pp;
    oE = 2 * vps * Pp;
    oB = 3 * vps * Pp;
    oC = 4 * vps * Pp;
    oCl = oC + vps * Pnp;
    n = oCl + (lo ? vps * Pnp : 0);
  }
};

// The schedule for a pattern whose incidence arrays (build_incidence's layout:
// psrc[pe], pdst[pe], in_off[pn + 1], in_q[pe], out_off[pn + 1], out_q[pe])
// are at pat, for stages of vps vertices.  Returns the terms per lane (a
// multiple of 4) and fills out[terms * 32]; 0 when the pattern takes the tile
// form (more than 64 pattern vertices or padded edge columns) or the stage is
// too large for the word's fields.
inline int vertex_warp_schedule(const int* pat, int pn, int pe, int pp, int pnp, int vps,
                                std::vector<uint32_t>* out) {
  out->clear();
  if (pn <= 0 || pn > 64 || pp > 64 || vps <= 0) return 0;
  const int ppl = pn <= 32 ? 1 : 2;
  const VwStage G(pp, pnp, false, vps);  // offsets of M, Y, CV (the same for FP32 and FP64)
  // every offset and slot must fit its field of the word
  if (G.oC + vps * pnp > 0x1000 || vps * (32 * ppl + 1) > 0x200) return 0;
  const int* inoff = pat + 2 * pe;
  const int* inq = inoff + pn + 1;
  const int* outoff = inq + pe;
  const int* outq = outoff + pn + 1;
  // jobs (jv, p), longest first (ties: jv, then p), each to the least loaded
  // lane (ties: the lowest)
  struct Job {
    int jv, p, len;
  };
  std::vector<Job> jobs;
  for (int jv = 0; jv < vps; ++jv)
    for (int p = 0; p < pn; ++p)
      jobs.push_back({jv, p, 1 + inoff[p + 1] - inoff[p] + outoff[p + 1] - outoff[p]});
  std::stable_sort(jobs.begin(), jobs.end(), [](const Job& x, const Job& y) { return x.len > y.len; });
  std::vector<std::vector<uint32_t>> lanes(32);
  for (const Job& j : jobs) {
    int best = 0;
    for (int l = 1; l < 32; ++l)
      if (lanes[l].size() < lanes[best].size()) best = l;
    std::vector<uint32_t>& L = lanes[best];
    const uint32_t slot = (uint32_t)(j.jv * (32 * ppl + 1) + j.p) << 16;
    std::vector<uint32_t> terms;
    terms.push_back((uint32_t)(G.oC + j.jv * pnp + j.p));  // -CV
    for (int i = inoff[j.p]; i < inoff[j.p + 1]; ++i)        // F[q], dst_q = p
      terms.push_back((uint32_t)(G.oM + j.jv * pp + inq[i]));
    for (int i = outoff[j.p]; i < outoff[j.p + 1]; ++i)      // R[q], src_q = p
      terms.push_back((uint32_t)(G.oY + j.jv * pp + outq[i]));
    terms.front() |= kSchedStart;
    terms.back() |= kSchedEnd;
    for (uint32_t& w : terms) L.push_back(w | slot);
  }
  size_t nt = 0;
  for (const auto& L : lanes) nt = std::max(nt, L.size());
  nt = (nt + 3) / 4 * 4;
  // padding terms (word 0) come after a lane's last job and change nothing it stores
  out->assign(nt * 32, 0u);
  for (int l = 0; l < 32; ++l)
    for (size_t t = 0; t < lanes[l].size(); ++t) (*out)[(t / 4) * 128 + l * 4 + t % 4] = lanes[l][t];
  return (int)nt;
}

}  // namespace acg
