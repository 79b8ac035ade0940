// acg_cdist_tc.cu -- the edge and vertex cost matrices on the 5th-generation
// tensor cores (tcgen05), for the mixed-precision path.
//
// dE[r][q] = ||x_r - y_q|| (ac.hxx:33-56, main.cu:110), and likewise dV
// (main.cu:109) with its per-column statistics, as ||x||^2 + ||y||^2 - 2 x.y, all
// three terms accumulated by the tensor cores: a [128 rows] x [N columns] x
// [K'] product per tile in TF32, with a three-term split that carries FP32
// accuracy in the cross term and the FP32 norms fed in as hi/lo TF32 pairs
// against ones (the operand layout is in acg_tc.cuh, dist_kp / dist_b_elem /
// dist_a_norms).  Both sides are first centred on the mean pattern feature
// vector m (distances do not change).  The norm form's error scales with
// ||x - m||^2 + ||y - m||^2, not with d^2, so a pair with
// 8 d^2 < ||x - m||^2 + ||y - m||^2 is recomputed exactly in the difference
// form from the FP32 features (dist_finish): near pairs (the planted ones) and
// data whose feature spread is large against the distances keep full FP32
// accuracy.  For N(0,1) features almost no pair is recomputed.  The edge phase
// that recomputes these costs in every iteration (acg_edge_tc.cu) uses the
// same operands and rule, so both give the same bits.
//
// One persistent CTA (8 warps) walks tiles of 128 data rows:
//   feature rows [128][kstride] FP32 --cp.async.bulk (TMA) + mbarrier--> smem
//     (double-buffered: the next tile's copy flies while this one computes)
//   threads split them into A' in the no-swizzle K-major core-matrix layout
//   thread 0 issues K'/8 MMAs into a TMEM accumulator, tcgen05.commit -> mbarrier
//   warps (lane quarter w % 4, column half w / 4) tcgen05.ld the accumulator,
//     form d and store their rows' 16-column chunks as 16-byte stores; for
//     the vertex matrix each lane also folds one column of the staged chunk
//     (16 of the warp's rows) into max(-d), LSE(d), LSE(-d) (main.cu:112,
//     116-117), merged per CTA in FP64 into the block partials at the end.
// Every mbarrier wait is bounded: on expiry the CTA records an error flag,
// waits (bounded) for its own operations in flight, frees its TMEM and exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "acg_cdist.cuh"
#include "acg_device.cuh"
#include "acg_tc.cuh"

namespace acg {

namespace {

using namespace tc;

constexpr int kTT = 256;               // threads per CTA
constexpr int kTM = 128;               // data rows per tile (the MMA's M)
constexpr int kStg = 20;  // staging row stride (floats): 16 columns + 16 bytes (no bank conflicts)

// Dynamic shared memory layout (byte offsets, each 128-aligned).
struct TcLayout {
  uint32_t a, b, x0, x1, y, nx, ny, mean, bar, tslot, total;
};
__host__ __device__ inline TcLayout tc_layout(int K, int kstride, int Pp, int N) {
  TcLayout L;
  (void)K;
  (void)Pp;
  const uint32_t kp = (uint32_t)dist_kp(kstride);  // K' padded to the MMA's K step
  uint32_t o = 0;
  // A' also holds the epilogue's staging rows (8 warps x 32 rows x kStg)
  const uint32_t abytes = (uint32_t)kTM * kp * 4, sbytes = (uint32_t)(kTT / 32) * 32 * kStg * 4;
  L.a = o;     o = al128(o + (abytes > sbytes ? abytes : sbytes));
  L.b = o;     o = al128(o + (uint32_t)N * kp * 4);
  L.x0 = o;    o = al128(o + (uint32_t)kTM * kstride * 4);
  L.x1 = o;    o = al128(o + (uint32_t)kTM * kstride * 4);
  L.y = o;     o = al128(o + (uint32_t)N * kstride * 4);
  L.nx = o;    o = al128(o + (uint32_t)kTM * 4);
  L.ny = o;    o = al128(o + (uint32_t)N * 4);
  L.mean = o;  o = al128(o + 32 * 4);
  L.bar = o;   o = al128(o + 3 * 8);
  L.tslot = o; o = al128(o + 4);
  L.total = o;
  return L;
}

struct TcArgs {
  const float* x;   // [nrows][KM] FP32 features (zero past K), in output row order
  const double* y;  // [P][K]
  float* out;       // [nrows][Pp]
  double* bpart;    // vertex matrix: block partials (StatSpec{P, 2P}), one column per CTA
  const int* rowmap;  // optional output row of each input row (null: the same row)
  float* outq;        // optional compact copy of columns [0, qcols) ([nrows][qcols]; qcols <= 16)
  int qcols;
  int* err;         // set to 1 when a bounded wait gave up
  long long nrows;
  int K, P, Pp, N, tcols;
};

// KM: the feature dimension padded to 4 (the FP32 row stride).  A' holds
// [x0 | x1 | x0 | norms] in blocks of KM columns, so each 4-wide core column
// comes from one block and is one 16-byte store.  STATS: the vertex matrix's
// column statistics.
template <int KM, bool STATS>
__global__ void __launch_bounds__(kTT, 3) cdist_tc_kernel(const TcArgs a) {
  constexpr int KP = dist_kp(KM);            // K' padded to the MMA's K step
  constexpr int KB = KM / 4;                // core columns per block
  extern __shared__ __align__(1024) unsigned char sm[];
  const TcLayout L = tc_layout(a.K, KM, a.Pp, a.N);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int K = a.K, P = a.P, Pp = a.Pp, N = a.N;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  float* sA = reinterpret_cast<float*>(sm + L.a);
  float* sB = reinterpret_cast<float*>(sm + L.b);
  float* sY = reinterpret_cast<float*>(sm + L.y);
  float* snx = reinterpret_cast<float*>(sm + L.nx);
  float* sny = reinterpret_cast<float*>(sm + L.ny);
  float* smean = reinterpret_cast<float*>(sm + L.mean);
  const uint32_t bar[3] = {sb + L.bar, sb + L.bar + 8, sb + L.bar + 16};  // x buffers 0, 1; MMA
  const long long ntiles = (a.nrows + kTM - 1) / kTM;

  if (tid == 0) {
    mbar_init(bar[0], 1);
    mbar_init(bar[1], 1);
    mbar_init(bar[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    tmem_alloc(sb + L.tslot, (uint32_t)a.tcols);
    fence_before();
  }
  // the centre m (mean pattern feature vector, zero past K) and the FP32
  // pattern rows for the exact recompute
  for (int k = tid; k < KM; k += kTT) {
    float s = 0.f;
    if (k < K)
      for (int q = 0; q < P; ++q) s += (float)a.y[(size_t)q * K + k];
    smean[k] = k < K ? s / (float)P : 0.f;
  }
  for (int i = tid; i < N * KM; i += kTT) {
    const int q = i / KM, k = i - q * KM;
    sY[i] = (q < P && k < K) ? (float)a.y[(size_t)q * K + k] : 0.f;
  }
  __syncthreads();
  // the centred pattern norms, then B' (acg_tc.cuh); A' zeroed (its padding
  // columns stay zero)
  for (int q = tid; q < N; q += kTT) {
    float s = 0.f;
    if (q < P)
      for (int k = 0; k < KM; ++k) {
        const float yc = sY[(size_t)q * KM + k] - smean[k];
        s = fmaf(yc, yc, s);
      }
    sny[q] = s;
  }
  __syncthreads();
  for (int i = tid; i < N * KP; i += kTT) {
    const int q = i / KP, k = i - q * KP, kk = k % KM;
    const float yk = (q < P && k < 3 * KM) ? sY[(size_t)q * KM + kk] - smean[kk] : 0.f;
    const float v = dist_b_elem(yk, q < P ? sny[q] : 0.f, q < P, k, KM);
    *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sB) + kmaj_off(q, k, N)) = v;
  }
  for (int i = tid; i < kTM * KP; i += kTT) sA[i] = 0.f;
  for (int r = tid; r < kTM; r += kTT) snx[r] = 0.f;
  __syncthreads();
  fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + L.tslot);

  const uint32_t lboA = (kTM / 8) * 128, lboB = (uint32_t)(N / 8) * 128, sbo = 128;
  const uint32_t idesc = idesc_tf32(kTM, N);
  constexpr uint32_t rowb = (uint32_t)KM * 4;
  uint32_t ph[3] = {0u, 0u, 0u};
  bool pend[2] = {false, false};  // a bulk load into buffer i is in flight (uniform)
  bool pend_mma = false;
  bool ok = true;
  // column statistics of lane l: column c * 16 + (l & 15) of the warp's chunk
  // slot j (c = warp / 4 + 2 j), over rows (l / 16) * 16 .. +15 of its 32
  constexpr int kSlots = STATS ? 4 : 1;
  float cmx[kSlots];
  OnlineLse<float> cl1[kSlots], cl2[kSlots];
#pragma unroll
  for (int j = 0; j < kSlots; ++j) {
    cmx[j] = -CUDART_INF_F;
    cl1[j].init();
    cl2[j].init();
  }

  long long tile = blockIdx.x;
  if (tile < ntiles) {
    if (tid == 0) {
      const int nr = (int)min((long long)kTM, a.nrows - tile * kTM);
      bulk_load(sb + L.x0, a.x + (size_t)tile * kTM * KM, (uint32_t)nr * rowb, bar[0]);
    }
    pend[0] = true;
  }
  for (int it = 0; tile < ntiles; tile += gridDim.x, ++it) {
    const int buf = it & 1;
    const uint32_t xoff = buf ? L.x1 : L.x0;
    const long long r0 = tile * kTM;
    const int nr = (int)min((long long)kTM, a.nrows - r0);
    // the next tile's features into the other buffer (its readers are done:
    // the barrier at the end of the previous iteration)
    const long long nt = tile + gridDim.x;
    if (nt < ntiles) {
      if (tid == 0) {
        const int nn = (int)min((long long)kTM, a.nrows - nt * kTM);
        fence_proxy_async();
        bulk_load(sb + (buf ? L.x0 : L.x1), a.x + (size_t)nt * kTM * KM, (uint32_t)nn * rowb,
                  bar[buf ^ 1]);
      }
      pend[buf ^ 1] = true;
    }
    ok = mbar_wait(bar[buf], ph[buf]);
    if (!__syncthreads_and(ok)) break;
    ph[buf] ^= 1u;
    pend[buf] = false;
    const float* sXb = reinterpret_cast<const float*>(sm + xoff);
    // split: thread (row r, half h): h = 0 writes the x0 blocks and the norm,
    // h = 1 the x1 block; one 16-byte store per core column
    {
      const int r = tid & (kTM - 1), h = tid >> 7;
      if (r < nr) {
        const float4* xr = reinterpret_cast<const float4*>(sXb + (size_t)r * KM);
        unsigned char* A = reinterpret_cast<unsigned char*>(sA);
        const uint32_t rb = (uint32_t)((r >> 3) * 128 + (r & 7) * 16);
        float s = 0.f;
#pragma unroll
        for (int j = 0; j < KB; ++j) {
          const float4 xv = xr[j];
          const float4 mv = reinterpret_cast<const float4*>(smean)[j];
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
            *reinterpret_cast<float4*>(A + (uint32_t)j * lboA + rb) = v0;
            *reinterpret_cast<float4*>(A + (uint32_t)(2 * KB + j) * lboA + rb) = v0;
          } else {
            *reinterpret_cast<float4*>(A + (uint32_t)(KB + j) * lboA + rb) =
                make_float4(h1[0], h1[1], h1[2], h1[3]);
          }
        }
        if (h == 0) {
          snx[r] = s;
          *reinterpret_cast<float4*>(A + (uint32_t)(3 * KB) * lboA + rb) = dist_a_norms(s);
        }
      }
    }
    fence_proxy_async();  // the generic-proxy writes of A' before the MMA reads them
    fence_before();
    __syncthreads();
    if (tid == 0) {
      fence_after();
#pragma unroll
      for (int st = 0; st < KP / 8; ++st)
        mma_tf32(tmem, smem_desc(sb + L.a + (uint32_t)st * 2 * lboA, lboA, sbo),
               smem_desc(sb + L.b + (uint32_t)st * 2 * lboB, lboB, sbo), idesc, st > 0);
      commit(bar[2]);
    }
    pend_mma = true;
    ok = mbar_wait(bar[2], ph[2]);
    if (!__syncthreads_and(ok)) break;
    ph[2] ^= 1u;
    pend_mma = false;
    fence_after();
    // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31 (its rows) and the
    // 16-column chunks c = w / 4, w / 4 + 2, ...; each chunk goes through the
    // warp's own staging rows (in A', idle until the next split) so that a
    // store instruction writes 8 rows x 64 contiguous bytes.  Leftover values
    // in A's zero-padding columns meet zero columns of B': they add nothing.
    {
      const int rw = (warp & 3) * 32, r = rw + lane;
      const float nx = snx[r];
      float* stg = sA + warp * 32 * kStg;  // [32][kStg], 16-column rows + padding
      // one chunk: d from the accumulator column values, staged, stored
      auto emit = [&](int c, const uint32_t (&v)[16], float& mx, OnlineLse<float>& l1,
                      OnlineLse<float>& l2) {
        float d[16];
#pragma unroll
        for (int j4 = 0; j4 < 4; ++j4) {
          const float4 ny4 = reinterpret_cast<const float4*>(sny + c * 16)[j4];
          const float nyv[4] = {ny4.x, ny4.y, ny4.z, ny4.w};
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            const int j = 4 * j4 + w, q = c * 16 + j;
            d[j] = (q < P && r < nr) ? dist_finish<KM>(__uint_as_float(v[j]), nx + nyv[w], sXb + (size_t)r * KM,
                                                       sY + (size_t)q * KM)
                                     : 0.f;
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
          *reinterpret_cast<float4*>(stg + lane * kStg + 4 * j) =
              make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
        __syncwarp();
        // lane t stores quarter t % 4 of row i * 8 + t / 4
        const int qt = lane & 3, col = c * 16 + qt * 4;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const int rr = i * 8 + (lane >> 2);
          if (rw + rr < nr && col < Pp) {
            const long long orow = a.rowmap ? (long long)__ldg(a.rowmap + r0 + rw + rr) : r0 + rw + rr;
            const float4 v4 = *reinterpret_cast<const float4*>(stg + rr * kStg + qt * 4);
            *reinterpret_cast<float4*>(a.out + (size_t)orow * Pp + col) = v4;
            if (col < a.qcols) *reinterpret_cast<float4*>(a.outq + (size_t)orow * a.qcols + col) = v4;
          }
        }
        if constexpr (STATS) {
          const int q = c * 16 + (lane & 15), h0 = (lane >> 4) * 16;
          if (q < P)
#pragma unroll 4
            for (int i = 0; i < 16; ++i) {
              if (rw + h0 + i >= nr) break;
              const float dv = stg[(h0 + i) * kStg + (lane & 15)];
              mx = fmaxf(mx, -dv);
              l1.add(dv);
              l2.add(-dv);
            }
        }
        __syncwarp();
      };
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int c = (warp >> 2) + 2 * j;
        if (c >= N / 16) break;
        uint32_t v[16];
        ld16(tmem + ((uint32_t)rw << 16) + (uint32_t)c * 16, v);
        wait_ld();
        emit(c, v, cmx[STATS ? j : 0], cl1[STATS ? j : 0], cl2[STATS ? j : 0]);
      }
    }
    fence_before();
    __syncthreads();  // TMEM read, this x buffer free
  }
  if (!ok) {
    // a wait gave up: record it, then wait (bounded) for what is in flight
    if (tid == 0) atomicExch(a.err, 1);
    for (int i = 0; i < 2; ++i)
      if (pend[i]) mbar_wait(bar[i], ph[i]);
    if (pend_mma) mbar_wait(bar[2], ph[2]);
  }
  if constexpr (STATS) {
    // block partials, one chunk slot at a time: column q's eight partials
    // (row quarters w % 4 of column half (q / 16) % 2, lane halves) merged in
    // a fixed order
    double* red = reinterpret_cast<double*>(sm + L.a);  // idle now: 256 x 5 doubles fit
    const int ncols = gridDim.x, col = blockIdx.x;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      if (32 * j >= P) break;
      __syncthreads();
      double* e = red + (size_t)tid * 5;
      e[0] = (double)cmx[j];
      e[1] = cl1[j].mval();
      e[2] = cl1[j].sval();
      e[3] = cl2[j].mval();
      e[4] = cl2[j].sval();
      __syncthreads();
      const int q = 32 * j + tid;
      if (tid < 32 && q < P) {
        double m = -CUDART_INF, am = -CUDART_INF, as = 0, bm = -CUDART_INF, bs = 0;
        const int wh = ((q >> 4) & 1) * 4;
        for (int wq = 0; wq < 4; ++wq)
          for (int h = 0; h < 2; ++h) {
            const double* x = red + (size_t)((wh + wq) * 32 + (q & 15) + 16 * h) * 5;
            m = fmax(m, x[0]);
            lse_merge(am, as, x[1], x[2]);
            lse_merge(bm, bs, x[3], x[4]);
          }
        a.bpart[(size_t)q * ncols + col] = m;
        a.bpart[(size_t)(P + 2 * q) * ncols + col] = am;
        a.bpart[(size_t)(P + 2 * q + 1) * ncols + col] = as;
        a.bpart[(size_t)(P + 2 * (P + q)) * ncols + col] = bm;
        a.bpart[(size_t)(P + 2 * (P + q) + 1) * ncols + col] = bs;
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, (uint32_t)a.tcols);
  }
}


// ---------------------------------------------------------------------------
// The edge matrix as a warp-specialised pipeline: one persistent CTA per SM,
// its tiles (blockIdx.x + i * gridDim.x) flowing through concurrent roles
//   issuer (1 thread)     feature rows [128][KM] by cp.async.bulk into a 3-slot
//                         ring (FFULL), three tiles ahead; once the split has
//                         filled an A' slot (ADONE) and the epilogue has freed
//                         an accumulator (ACCFREE): the tile's MMAs into one of
//                         four TMEM accumulators, commit -> MMA, then the copy
//                         of tile i + 3 into the slot the split has read
//   split (4 warps)       a thread per row: TF32 split into one of two A' slots
//                         and the row norm (NX, ADONE)
//   epilogue (2 x 8 warps) group g takes the tiles i = g mod 2; warp w: TMEM lane
//                         quarter w % 4, 16-column chunks of its column half;
//                         d as cdist_tc_kernel forms it (near pairs recomputed
//                         from the features in global memory), each chunk staged
//                         and stored as 8 rows x 64 bytes (rows through the
//                         optional row map; the first qcols columns also as
//                         compact rows of the outq copy), then ACCFREE
// so the split and MMAs run up to three tiles ahead of the epilogues, and each
// epilogue group has two tiles' time for one.  Same
// values as cdist_tc_kernel.  Bounded waits as there; a role whose wait gives
// up records the abort, the others leave at their next wait, and the copies and
// MMAs in flight are waited for before TMEM is freed.
constexpr int kWsSplit0 = 1, kWsSplitWarps = 4, kWsEpi0 = 5, kWsEpiWarps = 16;
constexpr int kWsT = (kWsEpi0 + kWsEpiWarps) * 32;  // 672 threads: at most 6 warps per SM sub-partition
constexpr int kWsAcc = 4;  // TMEM accumulators (and norm slots)
enum { W_FFULL = 0, W_ADONE = 3, W_MMA = 5, W_NX = 5 + kWsAcc, W_ACCFREE = 5 + 2 * kWsAcc,
       W_COUNT = 5 + 3 * kWsAcc };
enum { WM_ABORT = 0, WM_FISSUED = 1, WM_FWAITED = 2, WM_MISSUED = 3, WM_NYMAX = 4 /* float */ };

struct WsLayout {
  uint32_t a, b, f, stg, y, nx, ny, mean, misc, bar, tslot, total, aslot, fslot;
};
__host__ __device__ inline WsLayout ws_layout(int KM, int N) {
  WsLayout L;
  const uint32_t kp = (uint32_t)dist_kp(KM);
  L.aslot = (uint32_t)kTM * kp * 4;
  L.fslot = (uint32_t)kTM * (uint32_t)KM * 4;
  uint32_t o = 0;
  L.a = o;     o = al128(o + 2 * L.aslot);
  L.b = o;     o = al128(o + (uint32_t)N * kp * 4);
  L.f = o;     o = al128(o + 3 * L.fslot);
  L.stg = o;   o = al128(o + (uint32_t)kWsEpiWarps * 32 * kStg * 4);
  L.y = o;     o = al128(o + (uint32_t)N * KM * 4);
  L.nx = o;    o = al128(o + kWsAcc * kTM * 4);
  L.ny = o;    o = al128(o + (uint32_t)N * 4);
  L.mean = o;  o = al128(o + 32 * 4);
  L.misc = o;  o = al128(o + 8 * 4);
  L.bar = o;   o = al128(o + W_COUNT * 8);
  L.tslot = o; o = al128(o + 4);
  L.total = o;
  return L;
}

template <int KM>
__global__ void __launch_bounds__(kWsT, 1) cdist_ws_kernel(const TcArgs a) {
  constexpr int KP = dist_kp(KM);
  constexpr int KB = KM / 4;
  extern __shared__ __align__(1024) unsigned char sm[];
  const int K = a.K, P = a.P, Pp = a.Pp, N = a.N;
  const WsLayout L = ws_layout(KM, N);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sb = (uint32_t)__cvta_generic_to_shared(sm);
  float* sB = reinterpret_cast<float*>(sm + L.b);
  float* sY = reinterpret_cast<float*>(sm + L.y);
  float* snx = reinterpret_cast<float*>(sm + L.nx);
  float* sny = reinterpret_cast<float*>(sm + L.ny);
  float* smean = reinterpret_cast<float*>(sm + L.mean);
  int* smisc = reinterpret_cast<int*>(sm + L.misc);
  int* abort = smisc + WM_ABORT;
  auto bar = [&](int i) { return sb + L.bar + 8u * (uint32_t)i; };
  const long long ntiles = (a.nrows + kTM - 1) / kTM;
  if ((long long)blockIdx.x >= ntiles) return;  // before any barrier or TMEM: the whole CTA
  const int T = (int)((ntiles - 1 - blockIdx.x) / gridDim.x + 1);
  auto tile_of = [&](int it) { return (long long)blockIdx.x + (long long)it * gridDim.x; };
  auto rows_of = [&](int it) { return (int)min((long long)kTM, a.nrows - tile_of(it) * kTM); };

  if (tid == 0) {
    for (int i = 0; i < 3; ++i) mbar_init(bar(W_FFULL + i), 1);
    for (int i = 0; i < 2; ++i) mbar_init(bar(W_ADONE + i), kWsSplitWarps);
    for (int i = 0; i < kWsAcc; ++i) {
      mbar_init(bar(W_MMA + i), 1);
      mbar_init(bar(W_NX + i), kWsSplitWarps);
      mbar_init(bar(W_ACCFREE + i), kWsEpiWarps / 2);  // one epilogue group
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    for (int i = 0; i < 8; ++i) smisc[i] = 0;
  }
  if (warp == 0) {
    tmem_alloc(sb + L.tslot, (uint32_t)a.tcols);
    fence_before();
  }
  // the centre, the FP32 pattern rows, their centred norms and B' (as
  // cdist_tc_kernel); both A' slots zeroed (padding columns stay zero)
  for (int k = tid; k < KM; k += kWsT) {
    float s = 0.f;
    if (k < K)
      for (int q = 0; q < P; ++q) s += (float)a.y[(size_t)q * K + k];
    smean[k] = k < K ? s / (float)P : 0.f;
  }
  for (int i = tid; i < N * KM; i += kWsT) {
    const int q = i / KM, k = i - q * KM;
    sY[i] = (q < P && k < K) ? (float)a.y[(size_t)q * K + k] : 0.f;
  }
  __syncthreads();
  for (int q = tid; q < N; q += kWsT) {
    float s = 0.f;
    if (q < P)
      for (int k = 0; k < KM; ++k) {
        const float yc = sY[(size_t)q * KM + k] - smean[k];
        s = fmaf(yc, yc, s);
      }
    sny[q] = s;
  }
  __syncthreads();
  if (tid == 0) {
    float m = 0.f;
    for (int q = 0; q < P; ++q) m = fmaxf(m, sny[q]);
    reinterpret_cast<float*>(smisc)[WM_NYMAX] = m;
  }
  for (int i = tid; i < N * KP; i += kWsT) {
    const int q = i / KP, k = i - q * KP, kk = k % KM;
    const float yk = (q < P && k < 3 * KM) ? sY[(size_t)q * KM + kk] - smean[kk] : 0.f;
    *reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(sB) + kmaj_off(q, k, N)) =
        dist_b_elem(yk, q < P ? sny[q] : 0.f, q < P, k, KM);
  }
  for (uint32_t i = tid; i < 2 * L.aslot / 4; i += kWsT) reinterpret_cast<float*>(sm + L.a)[i] = 0.f;
  fence_proxy_async();  // B' and the zeroed A' before any MMA reads them
  __syncthreads();
  fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + L.tslot);
  auto give_up = [&]() {
    if (atomicExch(abort, 1) == 0) atomicExch(a.err, 1);
  };

  auto load_tile = [&](int it) {  // one thread: tile it's feature rows into slot it % 3
    bulk_load(sb + L.f + (uint32_t)(it % 3) * L.fslot, a.x + (size_t)tile_of(it) * kTM * KM,
              (uint32_t)rows_of(it) * (uint32_t)KM * 4u, bar(W_FFULL + it % 3));
    smisc[WM_FISSUED] = it + 1;
  };
  if (warp == 0) {
    // ---------------- issuer: feature copies and MMAs
    if (lane == 0) {
      const uint32_t lboA = (kTM / 8) * 128, lboB = (uint32_t)(N / 8) * 128, sbo = 128;
      const uint32_t idesc = idesc_tf32(kTM, N);
      for (int it = 0; it < min(3, T); ++it) load_tile(it);
      for (int it = 0; it < T; ++it) {
        bool ok = wait_bar(bar(W_ADONE + (it & 1)), (uint32_t)((it >> 1) & 1), abort);
        if (ok && it >= kWsAcc) ok = wait_bar(bar(W_ACCFREE + (it & 3)), (uint32_t)(((it >> 2) - 1) & 1), abort);
        if (!ok) {
          give_up();
          break;
        }
        fence_after();
        const uint32_t acc = tmem + (uint32_t)(it & 3) * (uint32_t)N;
        const uint32_t aa = sb + L.a + (uint32_t)(it & 1) * L.aslot;
#pragma unroll
        for (int k8 = 0; k8 < KP / 8; ++k8)
          mma_tf32(acc, smem_desc(aa + (uint32_t)k8 * 2 * lboA, lboA, sbo),
                   smem_desc(sb + L.b + (uint32_t)k8 * 2 * lboB, lboB, sbo), idesc, k8 > 0);
        commit(bar(W_MMA + (it & 3)));
        smisc[WM_MISSUED] = it + 1;
        if (it + 3 < T) {
          fence_proxy_async();  // the split's reads of the slot (before its ADONE arrival) precede the copy
          load_tile(it + 3);
        }
      }
    }
  } else if (warp < kWsEpi0) {
    // ---------------- split: a row per thread
    const int r = tid - kWsSplit0 * 32;
    const uint32_t lboA = (kTM / 8) * 128;
    for (int it = 0; it < T; ++it) {
      bool ok = wait_bar(bar(W_FFULL + it % 3), (uint32_t)((it / 3) & 1), abort);
      // the MMAs of tile it - 2 have read this A' slot; the epilogue of tile
      // it - 4 is done with this norm slot
      if (ok && it >= 2) ok = wait_bar(bar(W_MMA + ((it - 2) & 3)), (uint32_t)(((it - 2) >> 2) & 1), abort);
      if (ok && it >= kWsAcc) ok = wait_bar(bar(W_ACCFREE + (it & 3)), (uint32_t)(((it >> 2) - 1) & 1), abort);
      ok = named_bar_and(1, kWsSplitWarps * 32, ok);  // the split threads leave together or not at all
      if (!ok) {
        give_up();
        break;
      }
      if (r == 0) smisc[WM_FWAITED] = it + 1;
      unsigned char* A = sm + L.a + (uint32_t)(it & 1) * L.aslot;
      if (r < rows_of(it)) {
        const float4* xr = reinterpret_cast<const float4*>(sm + L.f + (uint32_t)(it % 3) * L.fslot +
                                                           (uint32_t)r * (uint32_t)KM * 4u);
        const uint32_t rb = (uint32_t)((r >> 3) * 128 + (r & 7) * 16);
        float s = 0.f;
#pragma unroll
        for (int jj = 0; jj < KB; ++jj) {
          const float4 xv = xr[jj];
          const float4 mv = reinterpret_cast<const float4*>(smean)[jj];
          const float c[4] = {xv.x - mv.x, xv.y - mv.y, xv.z - mv.z, xv.w - mv.w};
          float h0[4], h1[4];
#pragma unroll
          for (int w = 0; w < 4; ++w) {
            h0[w] = tf32_round(c[w]);
            h1[w] = tf32_round(c[w] - h0[w]);
            s = fmaf(c[w], c[w], s);
          }
          const float4 v0 = make_float4(h0[0], h0[1], h0[2], h0[3]);
          *reinterpret_cast<float4*>(A + (uint32_t)jj * lboA + rb) = v0;
          *reinterpret_cast<float4*>(A + (uint32_t)(2 * KB + jj) * lboA + rb) = v0;
          *reinterpret_cast<float4*>(A + (uint32_t)(KB + jj) * lboA + rb) = make_float4(h1[0], h1[1], h1[2], h1[3]);
        }
        snx[(it & 3) * kTM + r] = s;
        *reinterpret_cast<float4*>(A + (uint32_t)(3 * KB) * lboA + rb) = dist_a_norms(s);
      } else {
        snx[(it & 3) * kTM + r] = 0.f;
      }
      fence_proxy_async();  // the generic-proxy writes of A' before the MMA reads them
      __syncwarp();
      if (lane == 0) {  // the warp's rows of A', its norms and its reads of the feature slot are done
        mbar_arrive(bar(W_ADONE + (it & 1)));
        mbar_arrive(bar(W_NX + (it & 3)));
      }
    }
  } else {
    // ---------------- epilogue: d for this warp's rows and chunks, stored
    const int e = warp - kWsEpi0, q4 = warp & 3, grp = e >> 3, ch = (e >> 2) & 1;
    const int r = q4 * 32 + lane;
    float* stg = reinterpret_cast<float*>(sm + L.stg) + e * 32 * kStg;
    const float nymax = reinterpret_cast<const float*>(smisc)[WM_NYMAX];
    for (int it = grp; it < T; it += 2) {
      bool ok = wait_bar(bar(W_MMA + (it & 3)), (uint32_t)((it >> 2) & 1), abort);
      if (ok) ok = wait_bar(bar(W_NX + (it & 3)), (uint32_t)((it >> 2) & 1), abort);
      if (!__all_sync(0xffffffffu, ok)) {
        if (lane == 0) give_up();
        break;
      }
      fence_after();
      const int nr = rows_of(it);
      const long long r0 = tile_of(it) * kTM;
      const float nx = snx[(it & 3) * kTM + r];
      const float thr = 0.125f * (nx + nymax);
      // output rows of the four rows this lane stores, i * 8 + lane / 4
      int orow[4];  // row indices fit 31 bits (the CSR positions are int)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const long long row = r0 + q4 * 32 + i * 8 + (lane >> 2);
        orow[i] = (q4 * 32 + i * 8 + (lane >> 2) < nr) ? (a.rowmap ? __ldg(a.rowmap + row) : (int)row) : -1;
      }
      const uint32_t tbase = tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(it & 3) * (uint32_t)N;
      for (int c = ch; c < N / 16; c += 2) {
        uint32_t v[16];
        ld16(tbase + (uint32_t)c * 16, v);
        wait_ld();
        float d[16];
        // every pair of the chunk far (8 min d2 > nx + max ny): d2 * rsqrt(d2);
        // otherwise the rule pair by pair (dist_finish)
        float mn = __uint_as_float(v[0]);
#pragma unroll
        for (int j = 1; j < 16; ++j) mn = fminf(mn, __uint_as_float(v[j]));
        if (mn > thr) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const float d2 = __uint_as_float(v[j]);
            d[j] = d2 * rsqrtf(d2);
          }
        } else {
          const float* xr = a.x + (size_t)(r0 + (r < nr ? r : 0)) * KM;  // rare: near pairs
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int q = c * 16 + j;
            d[j] = (q < P && r < nr) ? dist_finish<KM>(__uint_as_float(v[j]), nx + sny[q], xr, sY + (size_t)q * KM)
                                     : 0.f;
          }
        }
        if ((c + 1) * 16 > P) {  // the chunk holds padding columns: zeros there
#pragma unroll
          for (int j = 0; j < 16; ++j)
            if (c * 16 + j >= P) d[j] = 0.f;
        }
        // staged through the warp's rows so that a store writes 8 rows x 64 bytes
#pragma unroll
        for (int j = 0; j < 4; ++j)
          *reinterpret_cast<float4*>(stg + lane * kStg + 4 * j) =
              make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
        __syncwarp();
        // lane t stores quarter t % 4 of row i * 8 + t / 4
        const int qt = lane & 3, col = c * 16 + qt * 4;
        if (col < Pp) {
#pragma unroll
          for (int i = 0; i < 4; ++i)
            if (orow[i] >= 0)
              *reinterpret_cast<float4*>(a.out + (size_t)orow[i] * Pp + col) =
                  *reinterpret_cast<const float4*>(stg + (i * 8 + (lane >> 2)) * kStg + qt * 4);
        }
        if (c == 0 && col < a.qcols) {  // the covered columns' compact copy (qcols <= 16: chunk 0)
#pragma unroll 1
          for (int i = 0; i < 4; ++i) {
            const int rr = q4 * 32 + i * 8 + (lane >> 2);
            if (rr < nr) {  // the output row again (no register kept live for it)
              const long long row = r0 + rr;
              const long long o = a.rowmap ? (long long)__ldg(a.rowmap + row) : row;
              *reinterpret_cast<float4*>(a.outq + (size_t)o * a.qcols + col) =
                  *reinterpret_cast<const float4*>(stg + (i * 8 + (lane >> 2)) * kStg + qt * 4);
            }
          }
        }
        __syncwarp();
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(bar(W_ACCFREE + (it & 3)));  // the accumulator and the norm slot are free
    }
  }
  __syncthreads();
  if (ld_volatile(abort)) {
    // copies and MMAs issued and not waited for land before the CTA leaves
    // (at most three feature copies and the last commit on each accumulator;
    // bounded waits)
    if (tid == 0)
      for (int it = smisc[WM_FWAITED]; it < smisc[WM_FISSUED]; ++it)
        mbar_wait(bar(W_FFULL + it % 3), (uint32_t)((it / 3) & 1));
    if (tid == 0)
      for (int it = max(0, smisc[WM_MISSUED] - kWsAcc); it < smisc[WM_MISSUED]; ++it)
        mbar_wait(bar(W_MMA + (it & 3)), (uint32_t)((it >> 2) & 1));
    fence_before();
    __syncthreads();
  }
  if (warp == 0) {
    fence_after();
    tmem_dealloc(tmem, (uint32_t)a.tcols);
  }
}

}  // namespace

bool cdist_tc_eligible(int K, int kstride, int P, int Pp) {
  const int N = (Pp + 15) / 16 * 16;
  return P > 0 && K >= 1 && K <= 32 && kstride == (K + 3) / 4 * 4 && N <= 128;
}

template <int KM, bool STATS>
static acg_status launch_tc(const TcArgs& a, int num_sms, int max_grid, int* grid_used, cudaStream_t s) {
  const TcLayout L = tc_layout(a.K, KM, a.Pp, a.N);
  auto* fn = cdist_tc_kernel<KM, STATS>;
  ACG_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
  ACG_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  // resident CTAs per SM from shared memory, registers and TMEM (512 columns)
  int dev = 0, smem_sm = 0, resv = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
  cudaDeviceGetAttribute(&resv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
  cudaFuncAttributes fa{};
  ACG_CUDA_TRY(cudaFuncGetAttributes(&fa, fn));
  const int regs = (fa.numRegs + 7) / 8 * 8;
  int nb = smem_sm / (int)(L.total + resv);
  nb = std::min(nb, 65536 / std::max(1, regs * kTT));
  nb = std::max(1, std::min(nb, 512 / a.tcols));
  const long long ntiles = (a.nrows + kTM - 1) / kTM;
  long long grid = std::min<long long>(ntiles, (long long)num_sms * nb);
  if (max_grid > 0) grid = std::min<long long>(grid, max_grid);
  grid = std::max<long long>(grid, 1);  // a CTA with no tile still writes empty partials
  fn<<<(int)grid, kTT, L.total, s>>>(a);
  ACG_LAUNCH_CHECK();
  if (grid_used) *grid_used = (int)grid;
  return ACG_OK;
}

template <bool STATS>
static acg_status launch_km(const TcArgs& a, int kstride, int num_sms, int max_grid, int* grid_used,
                            cudaStream_t s) {
  switch (kstride) {
    case 4: return launch_tc<4, STATS>(a, num_sms, max_grid, grid_used, s);
    case 8: return launch_tc<8, STATS>(a, num_sms, max_grid, grid_used, s);
    case 12: return launch_tc<12, STATS>(a, num_sms, max_grid, grid_used, s);
    case 16: return launch_tc<16, STATS>(a, num_sms, max_grid, grid_used, s);
    case 20: return launch_tc<20, STATS>(a, num_sms, max_grid, grid_used, s);
    case 24: return launch_tc<24, STATS>(a, num_sms, max_grid, grid_used, s);
    case 28: return launch_tc<28, STATS>(a, num_sms, max_grid, grid_used, s);
    default: return launch_tc<32, STATS>(a, num_sms, max_grid, grid_used, s);
  }
}

static TcArgs tc_args(const float* x, int K, const double* y, int P, int Pp, float* out, double* bpart,
                      long long nrows, int* err, const int* rowmap = nullptr, float* outq = nullptr,
                      int qcols = 0) {
  TcArgs a;
  a.rowmap = rowmap;
  a.outq = outq;
  a.qcols = outq ? qcols : 0;
  a.x = x;
  a.y = y;
  a.out = out;
  a.bpart = bpart;
  a.err = err;
  a.nrows = nrows;
  a.K = K;
  a.P = P;
  a.Pp = Pp;
  a.N = (Pp + 15) / 16 * 16;
  a.tcols = a.N <= 32 ? 32 : (a.N <= 64 ? 64 : 128);
  return a;
}

template <int KM>
static acg_status launch_ws(const TcArgs& a0, int num_sms, cudaStream_t s) {
  TcArgs a = a0;
  a.tcols = kWsAcc * a.N <= 32 ? 32 : (kWsAcc * a.N <= 64 ? 64 : (kWsAcc * a.N <= 128 ? 128 : (kWsAcc * a.N <= 256 ? 256 : 512)));
  const WsLayout L = ws_layout(KM, a.N);
  ACG_CUDA_TRY(cudaFuncSetAttribute(cdist_ws_kernel<KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total));
  const long long ntiles = (a.nrows + kTM - 1) / kTM;
  const int grid = (int)std::min<long long>(ntiles, (long long)num_sms);
  cdist_ws_kernel<KM><<<grid, kWsT, L.total, s>>>(a);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

// The warp-specialised edge matrix when its shared memory fits the device.
static bool ws_fits(int kstride, int N) {
  static int optin = -1;
  if (optin < 0) {
    int dev = 0;
    optin = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      optin = 0;
  }
  return ws_layout(kstride, N).total <= (uint32_t)optin;
}

acg_status launch_cdist_edges_tc(const float* x, int kstride, int K, const double* y, int P, int Pp,
                                 float* out, long long nrows, int* err, int num_sms, cudaStream_t s,
                                 const int* rowmap, float* outq, int qcols) {
  if (P == 0 || nrows == 0) return ACG_OK;
  if (!cdist_tc_eligible(K, kstride, P, Pp))
    return set_error(ACG_ERR_UNSUPPORTED, "tensor-core cdist: K=%d, %d columns", K, P);
  if (outq && (qcols % 4 || qcols > 16 || qcols > Pp))
    return set_error(ACG_ERR_INVALID_ARGUMENT, "tensor-core cdist: compact copy of %d columns", qcols);
  const TcArgs a = tc_args(x, K, y, P, Pp, out, nullptr, nrows, err, rowmap, outq, qcols);
  if (ws_fits(kstride, a.N)) {
    switch (kstride) {
      case 4: return launch_ws<4>(a, num_sms, s);
      case 8: return launch_ws<8>(a, num_sms, s);
      case 12: return launch_ws<12>(a, num_sms, s);
      case 16: return launch_ws<16>(a, num_sms, s);
      case 20: return launch_ws<20>(a, num_sms, s);
      case 24: return launch_ws<24>(a, num_sms, s);
      case 28: return launch_ws<28>(a, num_sms, s);
      default: return launch_ws<32>(a, num_sms, s);
    }
  }
  return launch_km<false>(a, kstride, num_sms, 0, nullptr, s);
}

acg_status launch_cdist_vertex_tc(const float* x, int kstride, int K, const double* y, int P, int Pp,
                                  float* out, double* bpart, long long nrows, int max_grid, int* grid_used,
                                  int* err, int num_sms, cudaStream_t s) {
  if (!cdist_tc_eligible(K, kstride, P, Pp))
    return set_error(ACG_ERR_UNSUPPORTED, "tensor-core vertex cdist: K=%d, %d columns", K, P);
  return launch_km<true>(tc_args(x, K, y, P, Pp, out, bpart, nrows, err), kstride, num_sms, max_grid,
                         grid_used, s);
}

}  // namespace acg
