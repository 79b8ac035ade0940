// acg_edge_tc.cu -- the edge phase of an FP32 BP iteration with the edge costs
// recomputed on the tensor cores instead of read from a stored cost matrix.
//
// It computes what edge_max_kernel computes from dE (ac.hxx:115-149 via
// main.cu:207-224, restructured as the segmented maximum over the
// destination-sorted CSR):
//     M[v][q] = max_{e in in(v)} z[s_e][q] - d(e, q),   d(e, q) = ||x_e - y_q||
// but forms d from the FP32 edge features (dst-CSR order, [De][KM]) and the
// pattern's edge features, with exactly the arithmetic of cdist_tc_kernel
// (acg_cdist_tc.cu): the centred TF32-split cross term on tcgen05.mma, the
// FP32 norms, d2 = fma(-2, cross, nx + ny), the exact difference-form
// recompute of near pairs (kNear * d2 < nx + ny), d = d2 * rsqrt(d2).  So M is
// the value the stored-matrix path gives, while the iteration reads ~76 bytes
// per in-edge (features, source and destination) instead of Pp * 4 + 4.
//
// One CTA per SM, 16 warps, tiles of 128 in-edges:
//   warps 0-7 (epilogue): tcgen05.ld the tile's accumulator (lane quarter
//     w % 4, 16-column chunks w / 4, w / 4 + 2, ...), form d, and overwrite the
//     tile's gathered z rows in shared memory with z[s_e] - d;
//   warps 8-15 (service): the segmented max of the previous tile (64 columns
//     x 4 groups of 32 rows, then the groups and the running segment merged),
//     the TF32 split of the next tile into A' and its MMA, the feature bulk
//     copies (cp.async.bulk, three tiles ahead) and the z-row gathers
//     (cp.async, two tiles ahead).
// The two halves work on different tiles, so each phase ends with one block
// barrier; the accumulator is double-buffered in TMEM, gathered rows in a
// three-slot ring.
// Work split: the tiles are cut into chunks of `tpc` consecutive tiles, dealt
// to the CTAs round-robin.  A vertex whose in-edges cross a chunk boundary
// leaves one partial row per chunk (the chunk it starts in: a tail row T; the
// others: a head row H); the CTA whose arrival completes the vertex's count
// takes their maximum into M (after a fence), and resets the count, so every
// launch leaves the counters at zero.  Maxima are exact, so the result does
// not depend on which CTA finishes.
// Every mbarrier wait is bounded: on expiry the CTA records an error flag,
// waits (bounded) for its copies and MMAs in flight, frees its TMEM and exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "acg_device.cuh"
#include "acg_iter.cuh"
#include "acg_tc.cuh"

namespace acg {

namespace {

using namespace tc;

constexpr int kET = 512;   // threads per CTA
constexpr int kTM = 128;   // in-edges per tile (the MMA's M)
constexpr int kEpi = 256;  // epilogue threads (warps 0-7); service threads follow
constexpr int kMaxCols = 64;
constexpr float kNear = 8.0f;  // cdist_tc_kernel's relative recompute threshold

inline __host__ __device__ int zstride_of(int Pp) { return Pp % 8 == 0 ? Pp + 4 : Pp; }

struct EtLayout {
  uint32_t a, b, f, z, dst, nx, y, ny, mean, hp, tp, gfl, misc, bar, tslot, total;
  int zstride;
  uint32_t zslot, fslot;
};
__host__ __device__ inline EtLayout et_layout(int KM, int N, int Pp) {
  EtLayout L;
  const uint32_t kp = (uint32_t)(3 * KM + 7) / 8 * 8;
  L.zstride = zstride_of(Pp);
  L.zslot = (uint32_t)kTM * (uint32_t)L.zstride * 4;
  L.fslot = (uint32_t)kTM * (uint32_t)KM * 4;
  uint32_t o = 0;
  L.a = o;     o = al128(o + (uint32_t)kTM * kp * 4);
  L.b = o;     o = al128(o + (uint32_t)N * kp * 4);
  L.f = o;     o = al128(o + 3 * L.fslot);
  L.z = o;     o = al128(o + 3 * L.zslot);
  L.dst = o;   o = al128(o + 3 * 130 * 4);
  L.nx = o;    o = al128(o + 2 * kTM * 4);
  L.y = o;     o = al128(o + (uint32_t)N * KM * 4);
  L.ny = o;    o = al128(o + (uint32_t)N * 4);
  L.mean = o;  o = al128(o + 32 * 4);
  L.hp = o;    o = al128(o + 4 * kMaxCols * 4);
  L.tp = o;    o = al128(o + 4 * kMaxCols * 4);
  L.gfl = o;   o = al128(o + 4 * 8 * 4);
  L.misc = o;  o = al128(o + 16 * 4);
  L.bar = o;   o = al128(o + 5 * 8);
  L.tslot = o; o = al128(o + 4);
  L.total = o;
  return L;
}

__device__ __forceinline__ void bar_service() {  // the 256 service threads
  asm volatile("bar.sync 1, 256;" ::: "memory");
}
__device__ __forceinline__ void bar_resolve() {  // service warps 8-9 (the column owners)
  asm volatile("bar.sync 2, 64;" ::: "memory");
}
__device__ __forceinline__ void cp16(uint32_t sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sdst), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }
__device__ __forceinline__ void cp_wait0() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Group flags written by the walk (one row of 8 ints per 32-row group).
enum { GF_NVALID = 0, GF_CONT, GF_HASEND, GF_TAILOPEN, GF_VFIRSTEND, GF_VLAST };

template <int KM>
__global__ void __launch_bounds__(kET, 1) edge_tc_kernel(const EdgeTcArgs a) {
  constexpr int KP = (3 * KM + 7) / 8 * 8;  // K' padded to the MMA's K step
  constexpr int KB = KM / 4;                // core columns per block
  extern __shared__ __align__(1024) unsigned char sm[];
  const int N = a.N, Pp = a.Pp, P = a.P, K = a.K;
  const EtLayout L = et_layout(KM, N, Pp);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool epi = tid < kEpi;
  const int st = tid - kEpi;  // service thread index (valid when !epi)
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  float* sA = reinterpret_cast<float*>(sm + L.a);
  float* sB = reinterpret_cast<float*>(sm + L.b);
  float* sZ = reinterpret_cast<float*>(sm + L.z);
  int* sDst = reinterpret_cast<int*>(sm + L.dst);
  float* snx = reinterpret_cast<float*>(sm + L.nx);
  float* sY = reinterpret_cast<float*>(sm + L.y);
  float* sny = reinterpret_cast<float*>(sm + L.ny);
  float* smean = reinterpret_cast<float*>(sm + L.mean);
  float* shp = reinterpret_cast<float*>(sm + L.hp);
  float* stp = reinterpret_cast<float*>(sm + L.tp);
  int* sgf = reinterpret_cast<int*>(sm + L.gfl);
  int* smisc = reinterpret_cast<int*>(sm + L.misc);
  const uint32_t fbar0 = sb + L.bar, mbar0 = sb + L.bar + 24;  // feature copies x3, MMAs x2
  const int zs = L.zstride;
  const long long De = a.De;
  const int tcols = a.tcols;

  // ---- this CTA's tiles: chunks b, b + G, ... of tpc tiles each
  const int G = (int)gridDim.x, b = (int)blockIdx.x, tpc = a.tpc;
  const int nmine = b < a.nchunks ? (a.nchunks - 1 - b) / G + 1 : 0;
  int n = nmine * tpc;
  if (nmine > 0 && b + (nmine - 1) * G == a.nchunks - 1) n -= tpc - (a.ntiles - (a.nchunks - 1) * tpc);
  auto chunk_of = [&](int j) { return b + (j / tpc) * G; };
  auto tile_of = [&](int j) { return chunk_of(j) * tpc + j % tpc; };
  auto rows_of = [&](int j) { return (int)min((long long)kTM, De - (long long)tile_of(j) * kTM); };
  auto chunk_last = [&](int j) { return j % tpc == tpc - 1 || j == n - 1; };

  if (tid == 0) {
    for (int i = 0; i < 3; ++i) mbar_init(fbar0 + 8 * i, 1);
    for (int i = 0; i < 2; ++i) mbar_init(mbar0 + 8 * i, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    smisc[8] = 0;  // a service thread's wait gave up (this phase)
  }
  if (warp == 0) {
    tmem_alloc(sb + L.tslot, (uint32_t)tcols);
    fence_before();
  }
  // the centre m, the FP32 pattern rows, B' and the centred pattern norms (as
  // cdist_tc_kernel); A' zeroed (its padding columns stay zero)
  for (int k = tid; k < KM; k += kET) {
    float s = 0.f;
    if (k < K)
      for (int q = 0; q < P; ++q) s += (float)a.y[(size_t)q * K + k];
    smean[k] = k < K ? s / (float)P : 0.f;
  }
  for (int i = tid; i < N * KM; i += kET) {
    const int q = i / KM, k = i - q * KM;
    sY[i] = (q < P && k < K) ? (float)a.y[(size_t)q * K + k] : 0.f;
  }
  __syncthreads();
  for (int i = tid; i < N * KP; i += kET) {
    const int q = i / KP, k = i - q * KP;
    float v = 0.f;
    if (k < 3 * KM) {
      const int blk = k / KM, kk = k - blk * KM;
      const float yc = q < P ? sY[(size_t)q * KM + kk] - smean[kk] : 0.f;
      const float y0 = tf32_round(yc);
      v = blk == 2 ? tf32_round(yc - y0) : y0;
    }
    *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sB) + kmaj_off(q, k, N)) = v;
  }
  for (int q = tid; q < N; q += kET) {
    float s = 0.f;
    if (q < P)
      for (int k = 0; k < KM; ++k) {
        const float yc = sY[(size_t)q * KM + k] - smean[k];
        s = fmaf(yc, yc, s);
      }
    sny[q] = s;
  }
  for (int i = tid; i < kTM * KP; i += kET) sA[i] = 0.f;
  for (int i = tid; i < 2 * kTM; i += kET) snx[i] = 0.f;
  fence_proxy_async();  // B' and the zeroed A' before any MMA reads them
  __syncthreads();
  fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + L.tslot);

  const uint32_t lboA = (kTM / 8) * 128, lboB = (uint32_t)(N / 8) * 128, sbo = 128;
  const uint32_t idesc = idesc_tf32(kTM, N);
  constexpr uint32_t rowb = (uint32_t)KM * 4;
  bool ok = true;
  // uniform progress counters: feature copies issued / waited, MMAs issued / waited
  int f_iss = 0, f_done = 0, m_iss = 0, m_done = 0;

  // ---- service-thread helpers
  // registers of the row loads two tiles ahead: the source of row st & 127,
  // the destination of row st - 1 (130 entries: the rows before and after)
  int rsrc = 0, rdst = -1;
  auto load_rows = [&](int j) {
    rsrc = 0;
    rdst = -1;
    if (j >= n) return;
    const long long r0 = (long long)tile_of(j) * kTM;
    const long long rs = r0 + (st & (kTM - 1));
    if (rs < De) rsrc = __ldg(a.src_of + rs);
    const long long rd = r0 - 1 + st;
    if (st < 130 && rd >= 0 && rd < De) rdst = __ldg(a.dst_of + rd);
  };
  // the gathered z rows of tile j into ring slot j % 3 (two threads per row)
  // and its destinations; always one commit group
  auto issue_rows = [&](int j) {
    if (j < n) {
      const int slot = j % 3;
      if (st < 130) sDst[slot * 130 + st] = rdst;
      const int r = st & (kTM - 1), h = st >> 7;
      const long long row = (long long)tile_of(j) * kTM + r;
      if (row < De) {
        const uint32_t dst = sb + L.z + (uint32_t)slot * L.zslot + (uint32_t)(r * zs) * 4;
        const float* src = a.z + (size_t)rsrc * Pp;
        const int nv = Pp / 4;
        for (int k = h; k < nv; k += 2) cp16(dst + 16 * k, src + 4 * k);
      }
    }
    cp_commit();
  };
  auto issue_feat = [&](int j) {  // one thread
    const long long r0 = (long long)tile_of(j) * kTM;
    fence_proxy_async();
    bulk_load(sb + L.f + (uint32_t)(j % 3) * L.fslot, a.x + (size_t)r0 * KM, (uint32_t)rows_of(j) * rowb,
              fbar0 + 8 * (j % 3));
  };
  // split of tile j's features into A' (thread (row r, half h): h = 0 the x0
  // blocks and the norm, h = 1 the x1 block)
  auto split = [&](int j) {
    const int r = st & (kTM - 1), h = st >> 7;
    if (r < rows_of(j)) {
      const float4* xr =
          reinterpret_cast<const float4*>(sm + L.f + (uint32_t)(j % 3) * L.fslot + (uint32_t)r * rowb);
      unsigned char* A = reinterpret_cast<unsigned char*>(sA);
      const uint32_t rb = (uint32_t)((r >> 3) * 128 + (r & 7) * 16);
      float s = 0.f;
#pragma unroll
      for (int jj = 0; jj < KB; ++jj) {
        const float4 xv = xr[jj];
        const float4 mv = reinterpret_cast<const float4*>(smean)[jj];
        float c[4] = {xv.x - mv.x, xv.y - mv.y, xv.z - mv.z, xv.w - mv.w};
        float h0[4], h1[4];
#pragma unroll
        for (int w = 0; w < 4; ++w) {
          h0[w] = tf32_round(c[w]);
          h1[w] = tf32_round(c[w] - h0[w]);
          s = fmaf(c[w], c[w], s);
        }
        if (h == 0) {
          const float4 v0 = make_float4(h0[0], h0[1], h0[2], h0[3]);
          *reinterpret_cast<float4*>(A + (uint32_t)jj * lboA + rb) = v0;
          *reinterpret_cast<float4*>(A + (uint32_t)(2 * KB + jj) * lboA + rb) = v0;
        } else {
          *reinterpret_cast<float4*>(A + (uint32_t)(KB + jj) * lboA + rb) = make_float4(h1[0], h1[1], h1[2], h1[3]);
        }
      }
      if (h == 0) snx[(j & 1) * kTM + r] = s;
    }
  };
  // split + MMA of tile j (all service threads)
  auto produce = [&](int j) {
    bool w = mbar_wait(fbar0 + 8 * (j % 3), (uint32_t)((j / 3) & 1));  // features of tile j
    if (j >= 1) w = w && mbar_wait(mbar0 + 8 * ((j - 1) & 1), (uint32_t)(((j - 1) >> 1) & 1));  // A' free
    if (!w) smisc[8] = 1;
    if (w) split(j);
    fence_proxy_async();  // the generic-proxy writes of A' before the MMA reads them
    fence_before();
    bar_service();
    const bool all = smisc[8] == 0;
    if (st == 0 && all) {
      fence_after();
      const uint32_t acc = tmem + (uint32_t)(j & 1) * (uint32_t)N;
#pragma unroll
      for (int s = 0; s < KP / 8; ++s)
        mma_tf32(acc, smem_desc(sb + L.a + (uint32_t)s * 2 * lboA, lboA, sbo),
                 smem_desc(sb + L.b + (uint32_t)s * 2 * lboB, lboB, sbo), idesc, s > 0);
      commit(mbar0 + 8 * (j & 1));
    }
    return all;
  };

  // ---- running segment state of the column owners (service threads 0..63)
  const int col = st & (kMaxCols - 1), grp = st >> 6;
  float run = neg_inf<float>();
  bool open = false, rhead = false;
  int hv = -1, tv = -1;  // this chunk's head / tail vertex (pieces written)

  // ---- prologue: copies for tiles 0..2, rows of tiles 0 and 1, tile 0's MMA
  if (!epi) {
    if (st == 0)
      for (int j = 0; j < 3 && j < n; ++j) issue_feat(j);
    load_rows(0);
    issue_rows(0);
    load_rows(1);
    issue_rows(1);
    load_rows(2);
  }
  f_iss = min(n, 3);
  if (n > 0) {
    if (!epi && !produce(0)) ok = false;
    m_iss = 1;
    if (!epi) cp_wait1();
  }
  fence_before();
  ok = __syncthreads_and(ok);
  fence_after();
  if (ok && n > 0) f_done = 1;

  for (int p = 0; ok && p <= n; ++p) {
    if (epi) {
      // ---------------- epilogue of tile p
      if (p < n) {
        const bool w = mbar_wait(mbar0 + 8 * (p & 1), (uint32_t)((p >> 1) & 1));
        if (!w) {
          ok = false;
        } else {
          fence_after();
          const int q4 = warp & 3, r = q4 * 32 + lane, half = warp >> 2;
          const int nr = rows_of(p);
          const float nx = snx[(p & 1) * kTM + r];
          float* zrow = sZ + (size_t)(p % 3) * (L.zslot / 4) + (size_t)r * zs;
          const long long erow = (long long)tile_of(p) * kTM + r;
          for (int c = half; c < N / 16; c += 2) {
            uint32_t v[16];
            ld16(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(p & 1) * (uint32_t)N + (uint32_t)c * 16, v);
            wait_ld();
            if (r >= nr || c * 16 >= Pp) continue;
            float d2[16], sn[16];
            float chk = 1.f;
#pragma unroll
            for (int j4 = 0; j4 < 4; ++j4) {
              const float4 ny4 = reinterpret_cast<const float4*>(sny + c * 16)[j4];
              const float nyv[4] = {ny4.x, ny4.y, ny4.z, ny4.w};
#pragma unroll
              for (int w4 = 0; w4 < 4; ++w4) {
                const int jj = 4 * j4 + w4;
                sn[jj] = nx + nyv[w4];
                d2[jj] = fmaf(-2.f, __uint_as_float(v[jj]), sn[jj]);
                chk = fminf(chk, fmaf(-0.125f, sn[jj], d2[jj]));
              }
            }
            float d[16];
            if (chk > 0.f) {  // every pair far: d2 > 0, no recompute
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) d[jj] = d2[jj] * rsqrtf(d2[jj]);
            } else {  // cdist_tc_kernel's per-pair rule
              const float* xr = a.x + (size_t)erow * KM;
#pragma unroll
              for (int jj = 0; jj < 16; ++jj) {
                const int q = c * 16 + jj;
                float t2 = d2[jj];
                if (q < P && kNear * t2 < sn[jj]) {
                  const float* yq = sY + (size_t)q * KM;
                  float acc = 0.f;
#pragma unroll 1
                  for (int k = 0; k < KM; ++k) {
                    const float t = __ldg(xr + k) - yq[k];
                    acc = fmaf(t, t, acc);
                  }
                  t2 = acc;
                }
                t2 = fmaxf(t2, 0.f);
                d[jj] = q < P ? (t2 > 0.f ? t2 * rsqrtf(t2) : 0.f) : 0.f;
              }
            }
#pragma unroll
            for (int j4 = 0; j4 < 4; ++j4) {
              if (c * 16 + 4 * j4 < Pp) {
                float4* zp = reinterpret_cast<float4*>(zrow + c * 16 + 4 * j4);
                float4 zv = *zp;
                zv.x -= d[4 * j4];
                zv.y -= d[4 * j4 + 1];
                zv.z -= d[4 * j4 + 2];
                zv.w -= d[4 * j4 + 3];
                *zp = zv;
              }
            }
          }
        }
      }
    } else {
      // ---------------- service: reduce tile p - 1
      if (p >= 1) {
        const int j = p - 1;
        const int slot = j % 3, nr = rows_of(j);
        const int* dsts = sDst + slot * 130;
        const float* zt = sZ + (size_t)slot * (L.zslot / 4);
        const int j0 = grp * 32;
        const int nvalid = max(0, min(32, nr - j0));
        const int rj = j0 + lane;
        const bool valid = rj < nr;
        const int dv = dsts[1 + rj];
        const unsigned endm = __ballot_sync(0xffffffffu, valid && dv != dsts[2 + rj]);
        const unsigned startm = __ballot_sync(0xffffffffu, valid && dv != dsts[rj]);
        const bool cont = nvalid > 0 && !(startm & 1u);
        const bool tailopen = nvalid > 0 && !((endm >> (nvalid - 1)) & 1u);
        if (col < Pp) {
          float acc = neg_inf<float>();
          bool head = cont;
#pragma unroll 8
          for (int jj = 0; jj < 32; ++jj) {
            if (jj < nvalid) {
              acc = fmaxf(acc, zt[(j0 + jj) * zs + col]);
              if ((endm >> jj) & 1u) {
                if (head) {
                  shp[grp * kMaxCols + col] = acc;
                  head = false;
                } else {
                  a.M[(size_t)dsts[1 + j0 + jj] * Pp + col] = acc;
                }
                acc = neg_inf<float>();
              }
            }
          }
          if (tailopen) {
            if (head)
              shp[grp * kMaxCols + col] = acc;  // through: no end in the group
            else
              stp[grp * kMaxCols + col] = acc;
          }
        }
        if ((st & 63) == 0) {
          int* f = sgf + grp * 8;
          f[GF_NVALID] = nvalid;
          f[GF_CONT] = cont;
          f[GF_HASEND] = endm != 0u;
          f[GF_TAILOPEN] = tailopen;
          f[GF_VFIRSTEND] = endm ? dsts[1 + j0 + __ffs(endm) - 1] : -1;
          f[GF_VLAST] = nvalid > 0 ? dsts[j0 + nvalid] : -1;
        }
        bar_service();
        // merge the groups and the running segment (column owners)
        if (st < kMaxCols) {
          const int chunk = chunk_of(j);
          if (j % tpc == 0) {  // a chunk starts: a continuing segment is its head
            open = false;
            rhead = false;
            hv = tv = -1;
            if (sgf[GF_CONT]) {
              open = true;
              rhead = true;
              run = neg_inf<float>();
            }
          }
          auto finish = [&](float val, int v) {
            if (rhead) {
              if (col < Pp) a.H[(size_t)chunk * Pp + col] = val;
              hv = v;
            } else if (col < Pp) {
              a.M[(size_t)v * Pp + col] = val;
            }
          };
          int vlast = -1;
#pragma unroll
          for (int g = 0; g < 4; ++g) {
            const int* f = sgf + g * 8;
            if (f[GF_NVALID] == 0) break;
            vlast = f[GF_VLAST];
            if (f[GF_CONT]) {
              run = fmaxf(run, col < Pp ? shp[g * kMaxCols + col] : 0.f);
              if (f[GF_HASEND]) {
                finish(run, f[GF_VFIRSTEND]);
                open = false;
              }
            }
            if (!f[GF_CONT] || f[GF_HASEND]) {
              if (f[GF_TAILOPEN]) {
                run = col < Pp ? stp[g * kMaxCols + col] : 0.f;
                open = true;
                rhead = false;
              } else {
                open = false;
              }
            }
          }
          if (chunk_last(j)) {
            // the segment open at the chunk's end: a through row (it is the
            // chunk's head) or the chunk's tail
            if (open) {
              if (rhead) {
                if (col < Pp) a.H[(size_t)chunk * Pp + col] = run;
                hv = vlast;
              } else {
                if (col < Pp) a.T[(size_t)chunk * Pp + col] = run;
                tv = vlast;
              }
            }
            open = false;
            // arrivals: the CTA completing a vertex's count merges its rows
            __threadfence();
            bar_resolve();
            const int CR = tpc * kTM;
            if (st == 0) {
              int lh = 0, lt = 0, cah = 0, cbh = 0, cbt = 0;
              if (hv >= 0) {
                cah = __ldg(a.off + hv) / CR;
                cbh = (__ldg(a.off + hv + 1) - 1) / CR;
                lh = atomicAdd(a.cnt + cah, 1) == cbh - cah;
              }
              if (tv >= 0) {
                cbt = (__ldg(a.off + tv + 1) - 1) / CR;
                lt = atomicAdd(a.cnt + chunk, 1) == cbt - chunk;
              }
              smisc[0] = lh;
              smisc[1] = cah;
              smisc[2] = cbh;
              smisc[3] = lt;
              smisc[4] = cbt;
            }
            bar_resolve();
            const int lh = smisc[0], cah = smisc[1], cbh = smisc[2], lt = smisc[3], cbt = smisc[4];
            if (lh || lt) __threadfence();
            if (lh && col < Pp) {
              float m = __ldcg(a.T + (size_t)cah * Pp + col);
              for (int k = cah + 1; k <= cbh; ++k) m = fmaxf(m, __ldcg(a.H + (size_t)k * Pp + col));
              a.M[(size_t)hv * Pp + col] = m;
            }
            if (lt && col < Pp) {
              float m = __ldcg(a.T + (size_t)chunk * Pp + col);
              for (int k = chunk + 1; k <= cbt; ++k) m = fmaxf(m, __ldcg(a.H + (size_t)k * Pp + col));
              a.M[(size_t)tv * Pp + col] = m;
            }
            if (st == 0) {
              if (lh) a.cnt[cah] = 0;  // ready for the next launch
              if (lt) a.cnt[chunk] = 0;
            }
            hv = tv = -1;
          }
        }
      }
      // ---------------- service: rows of tile p + 2, features of tile p + 3,
      // split + MMA of tile p + 1
      issue_rows(p + 2);  // its slot (that of tile p - 1) was read above
      load_rows(p + 3);
      if (st == 0 && p + 3 < n) issue_feat(p + 3);
      if (p + 1 < n && !produce(p + 1)) ok = false;
      cp_wait1();  // the rows of tile p + 1
    }
    // uniform bookkeeping of what is in flight: copies and MMAs issued now,
    // waits counted as done once the phase has ended without a failure
    if (p + 3 < n) f_iss = p + 4;
    if (p + 1 < n) m_iss = p + 2;
    fence_before();
    ok = __syncthreads_and(ok);
    fence_after();
    if (ok) {
      if (p + 1 < n) f_done = p + 2;
      if (p < n) m_done = p + 1;
    }
    if (!epi && st == 0) smisc[8] = 0;
  }
  if (!ok) {
    // a wait gave up: record it, then wait (bounded) for what is in flight
    if (tid == 0) atomicExch(a.err, 1);
    for (int j = f_done; j < f_iss; ++j) mbar_wait(fbar0 + 8 * (j % 3), (uint32_t)((j / 3) & 1));
    for (int j = m_done; j < m_iss; ++j) mbar_wait(mbar0 + 8 * (j & 1), (uint32_t)((j >> 1) & 1));
  }
  cp_wait0();
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, (uint32_t)tcols);
  }
}

template <int KM>
acg_status launch_km(const EdgeTcArgs& a, int grid, cudaStream_t s) {
  const EtLayout L = et_layout(KM, a.N, a.Pp);
  ACG_CUDA_TRY(cudaFuncSetAttribute(edge_tc_kernel<KM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)L.total));
  edge_tc_kernel<KM><<<grid, kET, L.total, s>>>(a);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

}  // namespace

size_t edge_tc_smem(int kstride, int Pp) {
  const int N = (Pp + 15) / 16 * 16;
  return et_layout(kstride, N, Pp).total;
}

bool edge_tc_eligible(int K, int kstride, int P, int Pp) {
  if (P <= 0 || K < 1 || kstride != (K + 3) / 4 * 4 || kstride > 24 || Pp > kMaxCols || Pp % 4) return false;
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return false;
  return edge_tc_smem(kstride, Pp) <= (size_t)optin;
}

int edge_tc_tiles_per_chunk(long long De, int num_sms) {
  const long long ntiles = (De + kTM - 1) / kTM;
  return (int)std::max<long long>(4, std::min<long long>(32, ntiles / std::max(1, 16 * num_sms)));
}

acg_status launch_edge_tc(const EdgeTcArgs& a0, int num_sms, cudaStream_t s) {
  if (a0.De == 0 || a0.P == 0) return ACG_OK;
  EdgeTcArgs a = a0;
  a.N = (a.Pp + 15) / 16 * 16;
  a.tcols = 2 * a.N <= 32 ? 32 : (2 * a.N <= 64 ? 64 : 128);
  a.ntiles = (int)((a.De + kTM - 1) / kTM);
  a.nchunks = (a.ntiles + a.tpc - 1) / a.tpc;
  const int grid = std::min(num_sms, a.nchunks);
  switch (a.KM) {
    case 4: return launch_km<4>(a, grid, s);
    case 8: return launch_km<8>(a, grid, s);
    case 12: return launch_km<12>(a, grid, s);
    case 16: return launch_km<16>(a, grid, s);
    case 20: return launch_km<20>(a, grid, s);
    case 24: return launch_km<24>(a, grid, s);
    default: return set_error(ACG_ERR_UNSUPPORTED, "fused edge phase: feature stride %d", a.KM);
  }
}

}  // namespace acg

namespace acg {

namespace {
__global__ void csr_rows_kernel(const int* __restrict__ off, int n, int* __restrict__ dst_of) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int e1 = off[v + 1];
    for (int e = off[v]; e < e1; ++e) dst_of[e] = v;
  }
}
}  // namespace

acg_status launch_csr_rows(const int* off, int n, int* dst_of, cudaStream_t s) {
  if (n <= 0) return ACG_OK;
  const int blocks = std::min((n + 255) / 256, 4096);
  csr_rows_kernel<<<blocks, 256, 0, s>>>(off, n, dst_of);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

}  // namespace acg
