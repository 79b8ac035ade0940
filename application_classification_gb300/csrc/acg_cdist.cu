// acg_cdist.cu -- cost matrices (feature cdist) of the data graph against the
// pattern, SIMT, register-blocked.
//
// dist[r][q] = sqrt(sum_k (x_rk - y_qk)^2) in the difference form of
// ac.hxx:33-56 (so exact pairs give exactly 0), computed in T from features
// stored as F.  A block stages a tile of data rows and all pattern rows into
// shared memory transposed ([k][row]), and each thread accumulates an
// RB x QB block of pairs: per feature index it reads RB + QB values and does
// 2 * RB * QB flops, instead of two loads per flop.
//
// MODE_EDGE also accumulates, per pattern edge q, the log-sum-exp of -dE over
// the "covered" elements of the reference's RE/FE initial buffer (flat index
// q * De + e < Pn * Dn, main.cu:113-114).  MODE_VERTEX accumulates, per
// pattern vertex p, max(-dV), LSE(dV) and LSE(-dV) (main.cu:112,116-117).
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "acg_cdist.cuh"
#include "acg_device.cuh"

namespace acg {

namespace {

constexpr int kCT = 256;

__host__ __device__ inline size_t c16(size_t b) { return (b + 15) & ~size_t(15); }

struct CdistSmem {
  size_t y, x, red, total;
  __host__ __device__ CdistSmem(int K, int QT, int RT, int sz, int nstat) {
    size_t o = 0;
    y = o; o += c16((size_t)K * QT * sz);
    x = o; o += c16((size_t)K * RT * sz);
    red = o; o += c16(sizeof(double) * (size_t)kCT * nstat);  // one column slot at a time
    total = o;
  }
};

template <typename T, typename F, int RB, int QB, int MODE>
__global__ void __launch_bounds__(kCT, 2)
cdist_rb_kernel(const CdistRbArgs<T, F> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NST = MODE == kCdistEdge ? 2 : 5;  // per-column statistics slots
  const int K = a.K, P = a.P, Pp = a.Pp;
  const int QG = (P + QB - 1) / QB;  // column groups
  const int RG = kCT / QG;           // row groups
  const int QT = QG * QB, RT = RG * RB;
  const CdistSmem L(K, QT, RT, sizeof(T), NST);
  T* s_y = reinterpret_cast<T*>(smem + L.y);  // [K][QT]
  T* s_x = reinterpret_cast<T*>(smem + L.x);  // [K][RT]
  double* s_red = reinterpret_cast<double*>(smem + L.red);
  const int tid = threadIdx.x;
  for (int t = tid; t < K * QT; t += kCT) {
    const int k = t / QT, q = t % QT;
    s_y[t] = q < P ? (T)a.y[(size_t)q * K + k] : T(0);
  }
  const int qg = tid % QG, rg = tid / QG;
  const bool active = rg < RG;
  const int q0 = qg * QB;

  // statistics of this thread's columns (FP32 partials carry a Kahan term;
  // partials are combined in FP64)
  OnlineLse<T> l1[QB], l2[QB];
  T mx[QB];
#pragma unroll
  for (int j = 0; j < QB; ++j) {
    l1[j].init();
    l2[j].init();
    mx[j] = neg_inf<T>();
  }

  const long long nrows = a.nrows;
  for (long long r0 = (long long)blockIdx.x * RT; r0 < nrows; r0 += (long long)gridDim.x * RT) {
    __syncthreads();  // previous tile's x is consumed (and s_y is written)
    const int rt = (int)min((long long)RT, nrows - r0);
    for (int t = tid; t < rt * K; t += kCT) {
      const int r = t / K, k = t % K;
      const long long row = a.row ? (long long)__ldg(a.row + r0 + r) : r0 + r;
      s_x[(size_t)k * RT + r] = (T)__ldg(a.x + (size_t)row * a.kstride + k);
    }
    __syncthreads();
    if (!active) continue;
    T acc[RB][QB];
#pragma unroll
    for (int i = 0; i < RB; ++i)
#pragma unroll
      for (int j = 0; j < QB; ++j) acc[i][j] = T(0);
    const int rb0 = rg * RB;
    for (int k = 0; k < K; ++k) {
      T xv[RB], yv[QB];
#pragma unroll
      for (int i = 0; i < RB; ++i) xv[i] = s_x[(size_t)k * RT + rb0 + i];
#pragma unroll
      for (int j = 0; j < QB; ++j) yv[j] = s_y[(size_t)k * QT + q0 + j];
#pragma unroll
      for (int i = 0; i < RB; ++i)
#pragma unroll
        for (int j = 0; j < QB; ++j) {
          const T d = xv[i] - yv[j];
          acc[i][j] += d * d;
        }
    }
#pragma unroll
    for (int i = 0; i < RB; ++i) {
      const long long r = r0 + rb0 + i;
      if (rb0 + i >= rt) break;
      // quirk coverage of this row's elements: q * De + e < lim  <=>  q < qlim
      int qlim = 0;
      if (MODE == kCdistEdge) {
        const long long e = a.eid ? (long long)__ldg(a.eid + r) : r;
        const long long room = a.lim - e;
        qlim = room <= 0 ? 0 : (int)min((long long)P, (room + a.De - 1) / a.De);
      }
      T dist[QB];
#pragma unroll
      for (int j = 0; j < QB; ++j) {
        const int q = q0 + j;
        dist[j] = q < P ? sqrt(acc[i][j]) : T(0);
        if (q < P) {
          if (MODE == kCdistEdge) {
            if (q < qlim) l1[j].add(-dist[j]);
          } else {
            mx[j] = fmax(mx[j], -dist[j]);
            l1[j].add(dist[j]);
            l2[j].add(-dist[j]);
          }
        }
      }
      // 16-byte stores of the row segment (columns beyond Pp are not stored)
      T* orow = a.out + (size_t)r * a.ostride + q0;
      constexpr int VW = 16 / sizeof(T);
#pragma unroll
      for (int j = 0; j < QB; j += VW) {
        if (q0 + j >= Pp) break;
        if constexpr (sizeof(T) == 4) {
          *reinterpret_cast<float4*>(orow + j) = make_float4(dist[j], dist[j + 1], dist[j + 2], dist[j + 3]);
        } else {
          *reinterpret_cast<double2*>(orow + j) = make_double2(dist[j], dist[j + 1]);
        }
      }
    }
  }
  // ---- block partials per column, row groups combined in order (one of the
  // QB columns of every thread at a time)
  if (a.bpart == nullptr) return;
  const int ncols = gridDim.x, col = blockIdx.x;
#pragma unroll
  for (int j = 0; j < QB; ++j) {
    __syncthreads();
    double* e = s_red + (size_t)tid * NST;
    if (MODE == kCdistEdge) {
      e[0] = l1[j].mval();
      e[1] = l1[j].sval();
    } else {
      e[0] = (double)mx[j];
      e[1] = l1[j].mval();
      e[2] = l1[j].sval();
      e[3] = l2[j].mval();
      e[4] = l2[j].sval();
    }
    __syncthreads();
    // one warp per column group: lanes merge row groups lane, lane + 32, ...,
    // then a fixed shuffle tree (the FP64 merges run in parallel)
    const int lane = tid & 31;
    for (int g = tid >> 5; g < QG; g += kCT / 32) {
      const int q = g * QB + j;
      if (q >= P) continue;  // uniform over the warp
      double m = -CUDART_INF, am = -CUDART_INF, as = 0, bm = -CUDART_INF, bs = 0;
      for (int r = lane; r < RG; r += 32) {
        const double* x = s_red + (size_t)(r * QG + g) * NST;
        if (MODE == kCdistEdge) {
          lse_merge(am, as, x[0], x[1]);
        } else {
          m = fmax(m, x[0]);
          lse_merge(am, as, x[1], x[2]);
          lse_merge(bm, bs, x[3], x[4]);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        lse_merge(am, as, __shfl_xor_sync(0xffffffffu, am, o), __shfl_xor_sync(0xffffffffu, as, o));
        if (MODE != kCdistEdge) {
          m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
          lse_merge(bm, bs, __shfl_xor_sync(0xffffffffu, bm, o), __shfl_xor_sync(0xffffffffu, bs, o));
        }
      }
      if (lane != 0) continue;
      if (MODE == kCdistEdge) {  // StatSpec{0, P}
        a.bpart[(size_t)(2 * q) * ncols + col] = am;
        a.bpart[(size_t)(2 * q + 1) * ncols + col] = as;
      } else {  // StatSpec{P, 2P}: max | lse(d) | lse(-d)
        a.bpart[(size_t)q * ncols + col] = m;
        a.bpart[(size_t)(P + 2 * q) * ncols + col] = am;
        a.bpart[(size_t)(P + 2 * q + 1) * ncols + col] = as;
        a.bpart[(size_t)(P + 2 * (P + q)) * ncols + col] = bm;
        a.bpart[(size_t)(P + 2 * (P + q) + 1) * ncols + col] = bs;
      }
    }
  }
}


// One thread per data row, for the edge cost matrix with K <= 32: the row's
// features in registers (KM = K rounded up to 4, zero padded: (0 - 0)^2 adds
// nothing), the pattern features in shared memory read as broadcast 16-byte
// loads, the distances of one row written by its thread as 16-byte stores (L2
// merges them into full lines).  No block-wide barrier after the prologue.
template <typename T, typename F, int KM>
__global__ void __launch_bounds__(kCT)
cdist_rows_kernel(const CdistRbArgs<T, F> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  T* s_y = reinterpret_cast<T*>(smem);  // [Pp][KM]
  const int K = a.K, P = a.P, Pp = a.Pp;
  for (int t = threadIdx.x; t < Pp * KM; t += kCT) {
    const int q = t / KM, k = t % KM;
    s_y[t] = (q < P && k < K) ? (T)a.y[(size_t)q * K + k] : T(0);
  }
  __syncthreads();
  constexpr int VW = 16 / sizeof(T);
  using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
  for (long long r = (long long)blockIdx.x * kCT + threadIdx.x; r < a.nrows;
       r += (long long)gridDim.x * kCT) {
    const long long src = a.row ? (long long)__ldg(a.row + r) : r;
    const F* xr = a.x + (size_t)src * a.kstride;
    T x[KM];
#pragma unroll
    for (int k = 0; k < KM; ++k) x[k] = k < K ? (T)__ldg(xr + k) : T(0);
    T* orow = a.out + (size_t)r * a.ostride;
    for (int q0 = 0; q0 < Pp; q0 += VW) {
      T d[VW];
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        const T* yq = s_y + (size_t)(q0 + j) * KM;
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < KM; k += VW) {
          const VT yv = *reinterpret_cast<const VT*>(yq + k);
#pragma unroll
          for (int w = 0; w < VW; ++w) {
            const T t = x[k + w] - reinterpret_cast<const T*>(&yv)[w];
            acc = fma(t, t, acc);
          }
        }
        d[j] = q0 + j < P ? sqrt(acc) : T(0);
      }
      if constexpr (sizeof(T) == 4)
        *reinterpret_cast<float4*>(orow + q0) = make_float4(d[0], d[1], d[2], d[3]);
      else
        *reinterpret_cast<double2*>(orow + q0) = make_double2(d[0], d[1]);
    }
  }
}
}  // namespace

// Register blocking per element type: FP32 4 rows x 8 columns, FP64 4 x 4.
template <typename T>
struct CdistBlock;
template <>
struct CdistBlock<float> {
  static constexpr int RB = 4, QB = 8;
};
template <>
struct CdistBlock<double> {
  static constexpr int RB = 4, QB = 4;
};

template <typename T, typename F>
size_t cdist_rb_smem(const CdistRbArgs<T, F>& a, int mode) {
  constexpr int RB = CdistBlock<T>::RB, QB = CdistBlock<T>::QB;
  const int QG = (a.P + QB - 1) / QB;
  const int RG = kCT / QG;
  return CdistSmem(a.K, QG * QB, RG * RB, sizeof(T), mode == kCdistEdge ? 2 : 5).total;
}

template <typename T, typename F>
acg_status launch_cdist_rb(const CdistRbArgs<T, F>& a, int mode, int blocks, cudaStream_t s) {
  constexpr int RB = CdistBlock<T>::RB, QB = CdistBlock<T>::QB;
  if (a.P == 0) return ACG_OK;  // no pattern columns: nothing to compute, no statistics
  const int QG = (a.P + QB - 1) / QB;
  if (QG > kCT) return set_error(ACG_ERR_UNSUPPORTED, "cdist: %d columns", a.P);
  const size_t sm = cdist_rb_smem(a, mode);
  if (mode == kCdistEdge) {
    if (sm > 48 * 1024)
      ACG_CUDA_TRY(cudaFuncSetAttribute(cdist_rb_kernel<T, F, RB, QB, kCdistEdge>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    cdist_rb_kernel<T, F, RB, QB, kCdistEdge><<<blocks, kCT, sm, s>>>(a);
  } else {
    if (sm > 48 * 1024)
      ACG_CUDA_TRY(cudaFuncSetAttribute(cdist_rb_kernel<T, F, RB, QB, kCdistVertex>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    cdist_rb_kernel<T, F, RB, QB, kCdistVertex><<<blocks, kCT, sm, s>>>(a);
  }
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}


#define ACG_ROWS_CASE(KM_)                                                                 \
  if (km == KM_) {                                                                         \
    const size_t sm = sizeof(T) * (size_t)a.Pp * KM_;                                      \
    if (sm > 48 * 1024)                                                                    \
      ACG_CUDA_TRY(cudaFuncSetAttribute(cdist_rows_kernel<T, F, KM_>,                      \
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)); \
    cdist_rows_kernel<T, F, KM_><<<blocks, kCT, sm, s>>>(a);                               \
    ACG_LAUNCH_CHECK();                                                                    \
    return ACG_OK;                                                                         \
  }

template <typename T, typename F>
acg_status launch_cdist_edges(const CdistRbArgs<T, F>& a, int blocks, cudaStream_t s) {
  if (a.P == 0 || a.nrows == 0) return ACG_OK;
  const int km = (a.K + 3) / 4 * 4;
  if (km >= 4) {
    ACG_ROWS_CASE(4) ACG_ROWS_CASE(8) ACG_ROWS_CASE(12) ACG_ROWS_CASE(16)
    ACG_ROWS_CASE(20) ACG_ROWS_CASE(24) ACG_ROWS_CASE(28) ACG_ROWS_CASE(32)
  }
  CdistRbArgs<T, F> b = a;  // wide features: the tiled kernel, no statistics
  b.bpart = nullptr;
  return launch_cdist_rb(b, kCdistEdge, blocks, s);
}

template acg_status launch_cdist_edges<double, double>(const CdistRbArgs<double, double>&, int, cudaStream_t);
template acg_status launch_cdist_edges<float, float>(const CdistRbArgs<float, float>&, int, cudaStream_t);

template acg_status launch_cdist_rb<double, double>(const CdistRbArgs<double, double>&, int, int, cudaStream_t);
template acg_status launch_cdist_rb<float, float>(const CdistRbArgs<float, float>&, int, int, cudaStream_t);

}  // namespace acg
