// acg_bp.cu -- the belief-propagation kernels of the matcher (SIMT part).
//
// Reference semantics (src/main.cu:107-247, src/ac.hxx:17-186), with pattern
// edge q = (src_q -> dst_q), data edge e = (s_e -> t_e), L(x) the row
// log-softmax over the data axis and CE = L(dE):
//   VF[q,v] = MU[dst_q,v] - FMax[q,v]          VR[q,v] = MU[src_q,v] - RMax[q,v]
//   RE[q,e] = VF[q,s_e] - CE[q,e]              FE[q,e] = VR[q,s_e] - CE[q,e]
//   RMax[q,v] = max(max_v' VF[q,v'], max_{e: s_e = v} L(RE)[q,e])
//   FMax[q,v] = max(max_v' VR[q,v'], max_{e: t_e = v} L(FE)[q,e])
//   MU[p,v] = L(-CV[p,v] + sum_{q: dst_q=p} FMax[q,v] + sum_{q: src_q=p} RMax[q,v])
//
// Both RE and FE gather at the edge's SOURCE (main.cu:184-185), so with
//   B[v,q]     = log sum_{e: s_e = v} exp(-dE[q,e])   (static)
//   dEmin[v,q] = min_{e: s_e = v} dE[q,e]             (static)
// the edge-sized work of an iteration collapses exactly to
//   log sum_e exp(RE[q,e]) = LSE_CE[q] + log sum_v exp(VF[q,v] + B[v,q])
//   max_{e: s_e = v} L(RE)  = VF[q,v] - dEmin[v,q] - log sum_v' exp(VF[q,v'] + B[v',q])
//   max_{e: t_e = v} L(FE)  = max_{e: t_e = v}(VR[q,s_e] - dE[q,e])
//                              - log sum_v' exp(VR[q,v'] + B[v',q])
// (LSE_CE cancels).  The only per-iteration edge work left is the segmented
// (max, -) reduction over each vertex's in-edges in the destination-sorted
// CSR, gathering the VR rows of the sources; no exp/log per edge remains.
//
// Global dependencies: each iteration needs column maxima / log-sum-exps of the
// previous VF, VR and MU.  They are carried unshifted: VF' = MU_raw[dst] -
// FMax, VR' = MU_raw[src] - RMax with MU_raw the un-normalised MU, and the
// previous column log-sum-exp S[p] of MU_raw is applied as a per-q constant
// (c_F[q] = S[dst_q], c_R[q] = S[src_q]):
//   RMax = max(mVF'[q] - c_F[q], VF'[v,q] - dEmin[v,q] - lR[q])
//   FMax = max(mVR'[q] - c_R[q], max_e(VR'[s_e,q] - dE[e,q]) - lF[q])
// with lR = LSE_v(VF' + B), lF = LSE_v(VR' + B).  So one fused kernel per
// iteration computes FMax, RMax, MU_raw and the next VF', VR' for each vertex,
// plus block partials of the next column statistics; stat_finalize combines
// those partials in a fixed order (results are deterministic).
#include <cuda_runtime.h>

#include <cstdint>

#include "acg_bp.cuh"
#include "acg_device.cuh"

namespace acg {

namespace {

template <typename T>
struct Vec;
template <>
struct Vec<double> {
  using type = double2;
  static constexpr int W = 2;
};
template <>
struct Vec<float> {
  using type = float4;
  static constexpr int W = 4;
};

template <typename T>
__device__ __forceinline__ T& lane_of(typename Vec<T>::type& v, int w) {
  return reinterpret_cast<T*>(&v)[w];
}
template <typename T>
__device__ __forceinline__ T lane_of(const typename Vec<T>::type& v, int w) {
  return reinterpret_cast<const T*>(&v)[w];
}

template <typename T>
__device__ __forceinline__ typename Vec<T>::type vzero() {
  typename Vec<T>::type z;
#pragma unroll
  for (int w = 0; w < Vec<T>::W; ++w) lane_of<T>(z, w) = T(0);
  return z;
}

// Shared-memory carving; the host computes sizes with the same rounding.
struct Carve {
  unsigned char* p;
  template <typename U>
  __device__ __forceinline__ U* take(size_t n) {
    U* r = reinterpret_cast<U*>(p);
    p += (n * sizeof(U) + 15) & ~size_t(15);
    return r;
  }
};
__host__ __device__ inline size_t carve_bytes(size_t n, size_t elem) {
  return (n * elem + 15) & ~size_t(15);
}

template <int G>
struct Grp {
  int lane, lig, gw;
  unsigned mask;
  __device__ __forceinline__ Grp() {
    lane = threadIdx.x & 31;
    lig = lane & (G - 1);
    gw = lane / G;
    mask = G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (gw * G));
  }
};

__device__ __forceinline__ double shfl_xor_d(double x, int o) {
  return __shfl_xor_sync(0xffffffffu, x, o);
}


// Combine, across the groups of a warp, values held by lanes with the same
// in-group index.  G == 32 is a no-op.
template <int G>
__device__ __forceinline__ double warp_group_max(double x) {
#pragma unroll
  for (int o = G; o < 32; o <<= 1) x = fmax(x, shfl_xor_d(x, o));
  return x;
}
template <int G>
__device__ __forceinline__ void warp_group_lse(double& m, double& s) {
#pragma unroll
  for (int o = G; o < 32; o <<= 1) {
    const double m2 = shfl_xor_d(m, o), s2 = shfl_xor_d(s, o);
    lse_merge(m, s, m2, s2);
  }
}

// After every warp wrote its per-slot values to red[warp][slot], combine the
// warps in order and write the block's partials [slot][ncols].
__device__ void block_partials_out(const double* red, int nwarps, StatSpec spec,
                                   double* bpart, int ncols, int col) {
  write_block_partials(red, nwarps, spec.nmax, spec.nlse, bpart, ncols, col);
}

// ------------------------------------------------------------- finalize
__global__ void __launch_bounds__(256)
stat_finalize_kernel(const double* __restrict__ bpart, int nblocks, StatSpec spec,
                     double* __restrict__ out) {
  __shared__ double sm[8], ss[8];
  const int o = blockIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (o < spec.nmax) {
    double m = -CUDART_INF;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) m = fmax(m, bpart[(size_t)o * nblocks + b]);
#pragma unroll
    for (int k = 16; k >= 1; k >>= 1) m = fmax(m, shfl_xor_d(m, k));
    if (lane == 0) sm[w] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      double r = sm[0];
      for (int k = 1; k < 8; ++k) r = fmax(r, sm[k]);
      out[o] = r;
    }
  } else {
    // two passes: the largest m of the non-empty partials, then the sum of
    // s_b exp(m_b - m) -- one independent exponential per partial; the sum
    // is taken in a fixed order (threads' strides, xor tree, warps in order)
    const int sl = spec.nmax + 2 * (o - spec.nmax);
    const double* pm = bpart + (size_t)sl * nblocks;
    const double* ps = bpart + (size_t)(sl + 1) * nblocks;
    double m = -CUDART_INF;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
      if (lse_nonempty(pm[b], ps[b])) m = fmax(m, pm[b]);
#pragma unroll
    for (int k = 16; k >= 1; k >>= 1) m = fmax(m, shfl_xor_d(m, k));
    if (lane == 0) sm[w] = m;
    __syncthreads();
    m = sm[0];
    for (int k = 1; k < 8; ++k) m = fmax(m, sm[k]);
    double s = 0.0;
    if (m > -CUDART_INF)
      for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
        if (lse_nonempty(pm[b], ps[b])) s += ps[b] * merge_exp(pm[b] - m, spec.f32 != 0);
#pragma unroll
    for (int k = 16; k >= 1; k >>= 1) s += shfl_xor_d(s, k);
    if (lane == 0) ss[w] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int k = 0; k < 8; ++k) t += ss[k];
      out[o] = (m > -CUDART_INF && t > 0.0) ? m + log(t) : -CUDART_INF;
    }
  }
}

// --------------------------------------------------------- the iteration
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kNPV = 4;  // pattern vertices per lane: Pn <= 4 * G

// dst[i][k] = (float)src[row ? row[i] : i][k], zero padding to kstride.
__global__ void convert_rows_kernel(const double* __restrict__ src, const int* __restrict__ row,
                                    long long n, int K, float* __restrict__ dst, int kstride) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * kstride) return;
  const long long i = t / kstride;
  const int k = (int)(t % kstride);
  float x = 0.f;
  if (k < K) x = __double2float_rn(src[(size_t)(row ? row[i] : i) * K + k]);
  dst[t] = x;
}

// Rows [e0, e1) of src (original edge order) as FP32, zero padded to kstride:
// into x32 in the same order and into dst at row pos[e].
__global__ void convert_scatter_kernel(const double* __restrict__ src, long long e0, long long e1, int K,
                                       const int* __restrict__ pos, float* __restrict__ x32,
                                       float* __restrict__ dst, int kstride) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (e1 - e0) * kstride) return;
  const long long e = e0 + t / kstride;
  const int k = (int)(t % kstride);
  const float x = k < K ? __double2float_rn(src[(size_t)e * K + k]) : 0.f;
  x32[(size_t)e * kstride + k] = x;
  dst[(size_t)__ldg(pos + e) * kstride + k] = x;
}

// pos[perm[r]] = r
__global__ void inverse_perm_kernel(const int* __restrict__ perm, long long n, int* __restrict__ pos) {
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) pos[perm[r]] = (int)r;
}

// ------------------------------------------------------ init vertex pass
// CV = dV - LSE_v(dV), MU0 = -dV - LSE_v(-dV) (main.cu:112,116-117);
// RMax0/FMax0 from the quirk buffer maxima (main.cu:113-114,119-120,135-146);
// then VF, VR of the first iteration (main.cu:165-176) and their statistics.
template <typename T, int G, int NQV>
__global__ void __launch_bounds__(kThreads)
init_vertex_kernel(const InitArgs<T> a) {
  constexpr int W = Vec<T>::W;
  constexpr int NQ = NQV * W;
  constexpr int GPB = kThreads / G;
  extern __shared__ __align__(16) unsigned char smem[];
  const int Pe = a.Pe, Pn = a.Pn, Pp = a.Pp;
  Carve cv{smem};
  int* s_pat = cv.take<int>(pattern_ints(Pn, Pe));
  double* s_lse1 = cv.take<double>(Pn);
  double* s_lse2 = cv.take<double>(Pn);
  double* s_vfmax0 = cv.take<double>(Pe);
  double* s_vrmax0 = cv.take<double>(Pe);
  double* s_lbuf = cv.take<double>(Pe);
  double* s_grp = cv.take<double>((size_t)GPB * Pn);
  double* s_red = cv.take<double>((size_t)kWarps * 6 * Pe);
  const int* s_psrc = s_pat;
  const int* s_pdst = s_pat + Pe;
  for (int t = threadIdx.x; t < pattern_ints(Pn, Pe); t += kThreads) s_pat[t] = a.pat[t];
  __syncthreads();
  for (int p = threadIdx.x; p < Pn; p += kThreads) {
    s_lse1[p] = a.gv[Pn + p];
    s_lse2[p] = a.gv[2 * Pn + p];
  }
  for (int q = threadIdx.x; q < Pe; q += kThreads) {
    s_vfmax0[q] = a.gv[s_pdst[q]] - a.gv[2 * Pn + s_pdst[q]];
    s_vrmax0[q] = a.gv[s_psrc[q]] - a.gv[2 * Pn + s_psrc[q]];
    // zeros of quirk row q: elements with flat index >= lim
    long long covered = a.qlim_col[q];
    covered = covered < 0 ? 0 : (covered > a.De ? a.De : covered);
    LseD r;  // LSE of the whole quirk row: covered part (ge) plus its zeros
    r.init();
    if (a.ge[q] > -CUDART_INF) r.merge(a.ge[q], 1.0);
    const long long zeros = a.De - covered;
    if (zeros > 0) r.merge(0.0, (double)zeros);
    s_lbuf[q] = r.value();
  }
  __syncthreads();
  const Grp<G> gr;
  const int gib = threadIdx.x / G;
  double* my_MU = s_grp + (size_t)gib * Pn;
  T mxF[NQ], mxR[NQ];
  OnlineLse<T> lr[NQ], lf[NQ];
#pragma unroll
  for (int k = 0; k < NQ; ++k) {
    mxF[k] = neg_inf<T>();
    mxR[k] = neg_inf<T>();
    lr[k].init();
    lf[k].init();
  }
  const int gstride = gridDim.x * GPB;
  for (int v = blockIdx.x * GPB + gib; v < a.Dn; v += gstride) {
    for (int p = gr.lig; p < Pn; p += G) {
      const double dv = (double)a.CV[(size_t)v * a.Pnp + p];
      const double c = dv - s_lse1[p];
      const T ch = (T)c;
      a.CV[(size_t)v * a.Pnp + p] = ch;
      if constexpr (sizeof(T) == 4) a.CVlo[(size_t)v * a.Pnp + p] = (T)(c - (double)ch);
      my_MU[p] = -dv - s_lse2[p];
    }
    __syncwarp(gr.mask);
    const int indeg = a.d_off[v + 1] - a.d_off[v];
    const int outdeg = a.s_off[v + 1] - a.s_off[v];
    const size_t vrow = (size_t)v * Pp;
#pragma unroll
    for (int k = 0; k < NQV; ++k)
#pragma unroll
      for (int w = 0; w < W; ++w) {
        const int q = (gr.lig + G * k) * W + w;
        if (q < Pp) {
          T y = T(0), r = T(0);
          if (q < Pe) {
            double R0 = s_vfmax0[q], F0 = s_vrmax0[q];
            const size_t qrow = (size_t)v * a.Pqc + q;
            if (outdeg > 0) R0 = fmax(R0, (q < a.qcov ? (double)a.Rq[qrow] : 0.0) - s_lbuf[q]);
            if (indeg > 0) F0 = fmax(F0, (q < a.qcov ? (double)a.Fq[qrow] : 0.0) - s_lbuf[q]);
            const double fd = my_MU[s_pdst[q]] - F0;
            const T f = (T)fd;
            r = (T)(my_MU[s_psrc[q]] - R0);
            y = (T)(fd - (double)a.dEmin[vrow + q]);  // no out-edges: -inf
            const T b = a.B[vrow + q];
            mxF[k * W + w] = fmax(mxF[k * W + w], f);
            mxR[k * W + w] = fmax(mxR[k * W + w], r);
            lr[k * W + w].add(f + b);
            lf[k * W + w].add(r + b);
          }
          a.vf[vrow + q] = y;
          a.vr[vrow + q] = r;
        }
      }
    __syncwarp(gr.mask);
  }
  const StatSpec spec{2 * Pe, 2 * Pe};
  const int slots = spec.slots();
  double* red = s_red + (size_t)(threadIdx.x >> 5) * slots;
#pragma unroll
  for (int k = 0; k < NQV; ++k)
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const int q = (gr.lig + G * k) * W + w;
      const double f = warp_group_max<G>((double)mxF[k * W + w]);
      const double r = warp_group_max<G>((double)mxR[k * W + w]);
      double m1 = lr[k * W + w].mval(), s1 = lr[k * W + w].sval();
      double m2 = lf[k * W + w].mval(), s2 = lf[k * W + w].sval();
      warp_group_lse<G>(m1, s1);
      warp_group_lse<G>(m2, s2);
      if (gr.gw == 0 && q < Pe) {
        red[q] = f;
        red[Pe + q] = r;
        red[spec.nmax + 2 * q] = m1;
        red[spec.nmax + 2 * q + 1] = s1;
        red[spec.nmax + 2 * (Pe + q)] = m2;
        red[spec.nmax + 2 * (Pe + q) + 1] = s2;
      }
    }
  __syncthreads();
  block_partials_out(s_red, kWarps, spec, a.bpart, gridDim.x, blockIdx.x);
}

__global__ void mu_output_kernel(double* __restrict__ mu, const double* __restrict__ S,
                                 long long n, int Pn) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) mu[i] -= S[i % Pn];
}

template <typename T>
size_t init_smem(GroupShape gs, int pn, int pe) {
  const int GPB = kThreads / gs.G;
  return carve_bytes(pattern_ints(pn, pe), sizeof(int)) + 2 * carve_bytes(pn, sizeof(double)) +
         3 * carve_bytes(pe, sizeof(double)) + carve_bytes((size_t)GPB * pn, sizeof(double)) +
         carve_bytes((size_t)kWarps * 6 * pe, sizeof(double));
}

// Dispatch over the instantiated group shapes.
#define ACG_SHAPES(X) \
  X(8, 1) X(16, 1) X(32, 1) X(32, 2) X(32, 3) X(32, 4)

template <typename T, typename F>
acg_status dispatch_shape(GroupShape gs, F&& f);

}  // namespace

GroupShape choose_shape(int elem_bytes, int pp, int pn) {
  const int W = 16 / elem_bytes;
  const int nvec = (pp + W - 1) / W;
  const int gmin_p = (pn + kNPV - 1) / kNPV;
  GroupShape gs{32, 1};
  for (int g : {8, 16, 32})
    if (g >= nvec && g >= gmin_p) {
      gs.G = g;
      gs.NQV = 1;
      return gs;
    }
  gs.G = 32;
  gs.NQV = (nvec + 31) / 32;
  return gs;
}

#define ACG_INIT_CASE(G_, N_)                                                           \
  if (gs.G == G_ && gs.NQV == N_) {                                                     \
    const size_t sm = init_smem<T>(gs, a.Pn, a.Pe);                                     \
    if (sm > 48 * 1024)                                                                 \
      cudaFuncSetAttribute(init_vertex_kernel<T, G_, N_>,                               \
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);       \
    init_vertex_kernel<T, G_, N_><<<blocks, kThreads, sm, s>>>(a);                      \
    ACG_LAUNCH_CHECK();                                                                 \
    return ACG_OK;                                                                      \
  }

template <typename T>
acg_status launch_init_vertex(const InitArgs<T>& a, GroupShape gs, int blocks, cudaStream_t s) {
  ACG_SHAPES(ACG_INIT_CASE)
  return set_error(ACG_ERR_UNSUPPORTED, "no init kernel for G=%d NQV=%d", gs.G, gs.NQV);
}

acg_status launch_finalize(const double* bpart, int nblocks, StatSpec spec, double* out,
                           cudaStream_t s) {
  const int n = spec.outs();
  if (n == 0) return ACG_OK;
  stat_finalize_kernel<<<n, 256, 0, s>>>(bpart, nblocks, spec, out);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

acg_status launch_convert_rows(const double* src, const int* row, long long n, int K, float* dst,
                               int kstride, cudaStream_t s) {
  const long long tot = n * kstride;
  if (tot == 0) return ACG_OK;
  convert_rows_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(src, row, n, K, dst, kstride);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

acg_status launch_convert_scatter(const double* src, long long e0, long long e1, int K, const int* pos,
                                  float* x32, float* dst, int kstride, cudaStream_t s) {
  const long long tot = (e1 - e0) * kstride;
  if (tot <= 0) return ACG_OK;
  convert_scatter_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(src, e0, e1, K, pos, x32, dst, kstride);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

acg_status launch_inverse_perm(const int* perm, long long n, int* pos, cudaStream_t s) {
  if (n == 0) return ACG_OK;
  inverse_perm_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(perm, n, pos);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

acg_status launch_mu_output(double* mu, const double* S, long long Dn, int Pn, cudaStream_t s) {
  const long long n = Dn * Pn;
  if (n == 0) return ACG_OK;
  mu_output_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(mu, S, n, Pn);
  ACG_LAUNCH_CHECK();
  return ACG_OK;
}

template acg_status launch_init_vertex<double>(const InitArgs<double>&, GroupShape, int, cudaStream_t);
template acg_status launch_init_vertex<float>(const InitArgs<float>&, GroupShape, int, cudaStream_t);

}  // namespace acg
