// acg_device.cuh -- device helpers shared by the matcher's kernels.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include <cstdint>

#include "acg_common.h"

#define ACG_CUDA_TRY(expr)                                                    \
  do {                                                                        \
    cudaError_t acg_e_ = (expr);                                              \
    if (acg_e_ != cudaSuccess)                                                \
      return acg::set_error(acg_e_ == cudaErrorMemoryAllocation               \
                                ? ACG_ERR_OUT_OF_MEMORY : ACG_ERR_CUDA,       \
                            "%s:%d: %s: %s", __FILE__, __LINE__, #expr,       \
                            cudaGetErrorString(acg_e_));                      \
  } while (0)

#define ACG_LAUNCH_CHECK()                                                    \
  do {                                                                        \
    cudaError_t acg_e_ = cudaGetLastError();                                  \
    if (acg_e_ != cudaSuccess)                                                \
      return acg::set_error(ACG_ERR_CUDA, "%s:%d: launch: %s", __FILE__,      \
                            __LINE__, cudaGetErrorString(acg_e_));            \
  } while (0)

namespace acg {

constexpr int kNumSMs = 152;  // GB300: 2 dies x 76 SMs

template <typename T>
__device__ __forceinline__ T neg_inf();
template <>
__device__ __forceinline__ double neg_inf<double>() { return -CUDART_INF; }
template <>
__device__ __forceinline__ float neg_inf<float>() { return -CUDART_INF_F; }

template <typename T>
__device__ __forceinline__ T pos_inf() { return -neg_inf<T>(); }

__device__ __forceinline__ double dev_exp(double x) { return exp(x); }
__device__ __forceinline__ float dev_exp(float x) { return expf(x); }
__device__ __forceinline__ double dev_log(double x) { return log(x); }
__device__ __forceinline__ float dev_log(float x) { return logf(x); }

// Running log-sum-exp over a stream of values: the sum of exp(x - m) for the
// largest value m seen so far.  The FP32 form keeps a Kahan compensation term
// so that a thread's partial sum carries only O(eps) relative error however
// many terms it adds; partials are combined in FP64 (LseD below).
template <typename T>
struct OnlineLse;

template <>
struct OnlineLse<double> {
  double m, s;
  __device__ __forceinline__ void init() {
    m = -CUDART_INF;
    s = 0.0;
  }
  __device__ __forceinline__ void add(double x) {
    if (!(x > -CUDART_INF)) return;
    if (x > m) {
      s = s * exp(m - x) + 1.0;
      m = x;
    } else {
      s += exp(x - m);
    }
  }
  // add x = hi + lo (lo tiny next to hi)
  __device__ __forceinline__ void add2(double hi, double lo) { add(hi + lo); }
  __device__ __forceinline__ void add2_fast(double hi, double lo) { add(hi + lo); }
  __device__ __forceinline__ void add_fast(double x) { add(x); }
  __device__ __forceinline__ double mval() const { return m; }
  __device__ __forceinline__ double sval() const { return s; }
};

template <>
struct OnlineLse<float> {
  float m, s, c;
  __device__ __forceinline__ void init() {
    m = -CUDART_INF_F;
    s = 0.f;
    c = 0.f;
  }
  __device__ __forceinline__ void kahan(float e) {
    float y = e - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ void add(float x) {
    if (!(x > -CUDART_INF_F)) return;
    if (x > m) {
      float sc = expf(m - x);
      s *= sc;
      c *= sc;
      m = x;
      kahan(1.f);
    } else {
      kahan(expf(x - m));
    }
  }
  // add x = hi + lo (lo tiny next to hi): exp(hi + lo - m) = exp(hi - m)(1 + lo)
  // to first order, so the low part of a compensated value is not lost
  __device__ __forceinline__ void add2(float hi, float lo) {
    if (!(hi > -CUDART_INF_F)) return;
    if (hi > m) {
      float sc = expf(m - hi);
      s *= sc;
      c *= sc;
      m = hi;
      kahan(1.f + lo);
    } else {
      kahan(expf(hi - m) * (1.f + lo));
    }
  }
  // add2 for finite hi, branch-free with the fast exponential (hot path)
  __device__ __forceinline__ void add2_fast(float hi, float lo) {
    const float mn = fmaxf(m, hi);
    const float sc = __expf(m - mn);  // m = -inf -> 0
    s *= sc;
    c *= sc;
    kahan(__expf(hi - mn) * (1.f + lo));
    m = mn;
  }
  // Branch-free variant with the fast exponential, for the hot per-vertex
  // statistics: m' = max(m, x); s = s e^(m - m') + e^(x - m').  Terms near the
  // running maximum dominate the sum and carry ~1e-7 relative error.
  __device__ __forceinline__ void add_fast(float x) {
    if (!(x > -CUDART_INF_F)) return;
    const float mn = fmaxf(m, x);
    const float sc = __expf(m - mn);  // m = -inf -> 0
    s *= sc;
    c *= sc;
    kahan(__expf(x - mn));
    m = mn;
  }
  // Four values at once (-inf entries add nothing): one rescale of the running
  // sum for the block's maximum, the four terms summed in FP32 first.
  __device__ __forceinline__ void add4_fast(float x0, float x1, float x2, float x3) {
    const float m4 = fmaxf(fmaxf(x0, x1), fmaxf(x2, x3));
    if (!(m4 > -CUDART_INF_F)) return;
    const float mn = fmaxf(m, m4);
    const float sc = __expf(m - mn);  // m = -inf -> 0
    s *= sc;
    c *= sc;
    kahan((__expf(x0 - mn) + __expf(x1 - mn)) + (__expf(x2 - mn) + __expf(x3 - mn)));
    m = mn;
  }
  // add2_fast of four compensated values hi + lo (hi = -inf: nothing)
  __device__ __forceinline__ void add2x4_fast(const float (&hi)[4], const float (&lo)[4]) {
    const float m4 = fmaxf(fmaxf(hi[0], hi[1]), fmaxf(hi[2], hi[3]));
    if (!(m4 > -CUDART_INF_F)) return;
    const float mn = fmaxf(m, m4);
    const float sc = __expf(m - mn);
    s *= sc;
    c *= sc;
    float e[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) e[i] = __expf(hi[i] - mn) * (1.f + lo[i]);
    kahan((e[0] + e[1]) + (e[2] + e[3]));
    m = mn;
  }
  __device__ __forceinline__ double mval() const { return (double)m; }
  __device__ __forceinline__ double sval() const { return (double)s - (double)c; }
};

// (max, scaled sum) pair in FP64 for combining partial log-sum-exps.
struct LseD {
  double m, s;
  __device__ __forceinline__ void init() {
    m = -CUDART_INF;
    s = 0.0;
  }
  __device__ __forceinline__ void merge(double m2, double s2) {
    if (!(m2 > -CUDART_INF) || s2 == 0.0) return;
    if (!(m > -CUDART_INF)) {
      m = m2;
      s = s2;
      return;
    }
    if (m2 > m) {
      s = s * exp(m - m2) + s2;
      m = m2;
    } else {
      s += s2 * exp(m2 - m);
    }
  }
  __device__ __forceinline__ double value() const {
    return (m > -CUDART_INF && s > 0.0) ? m + log(s) : -CUDART_INF;
  }
};

__device__ __forceinline__ void lse_merge(double& m, double& s, double m2, double s2) {
  LseD a{m, s};
  a.merge(m2, s2);
  m = a.m;
  s = a.s;
}

// exp(d) for d <= 0, the factor that rescales a partial sum when partial
// log-sum-exps are merged.  FP64 for FP64 statistics; the FP32 exponential
// (relative error ~1e-7, that of the FP32 partial sums it scales) for the
// statistics of FP32 kernels -- FP64 transcendentals are slow on this GPU.
__device__ __forceinline__ double merge_exp(double d, bool f32) {
  return f32 ? (double)expf((float)d) : exp(d);
}
// A partial (m, s) that holds no term: m = -inf or s = 0.
__device__ __forceinline__ bool lse_nonempty(double m, double s) {
  return m > -CUDART_INF && s != 0.0;
}

// Per-block statistics written as partials [slot][column]: `nmax` maxima, then
// `nlse` log-sum-exps as (m, s) pairs.  red[w * slots + slot] holds warp w's
// value; warps are combined in order, so the result does not depend on timing.
// Each log-sum-exp is merged in two passes (the largest m, then the sum of
// s_w exp(m_w - m)): one independent exponential per partial, no chain.
__device__ __forceinline__ void write_block_partials(const double* red, int nwarps, int nmax,
                                                     int nlse, double* bpart, int ncols,
                                                     int col, bool f32 = false) {
  const int slots = nmax + 2 * nlse;
  for (int j = threadIdx.x; j < nmax + nlse; j += blockDim.x) {
    if (j < nmax) {
      double m = -CUDART_INF;
      for (int w = 0; w < nwarps; ++w) m = fmax(m, red[w * slots + j]);
      bpart[(size_t)j * ncols + col] = m;
    } else {
      const int sm = nmax + 2 * (j - nmax);
      double m = -CUDART_INF, s = 0.0;
      for (int w = 0; w < nwarps; ++w) {
        const double m2 = red[w * slots + sm], s2 = red[w * slots + sm + 1];
        if (lse_nonempty(m2, s2)) m = fmax(m, m2);
      }
      if (m > -CUDART_INF) {
        for (int w = 0; w < nwarps; ++w) {
          const double m2 = red[w * slots + sm], s2 = red[w * slots + sm + 1];
          if (lse_nonempty(m2, s2)) s += s2 * merge_exp(m2 - m, f32);
        }
      }
      bpart[(size_t)sm * ncols + col] = m;
      bpart[(size_t)(sm + 1) * ncols + col] = s;
    }
  }
}

// Compensated running sum for FP32 (TwoSum: hi + lo carries the exact sum of
// the added terms to within one rounding); plain sum for FP64.
template <typename T>
struct CSum;
template <>
struct CSum<float> {
  float hi, lo;
  __device__ __forceinline__ void init(float x) {
    hi = x;
    lo = 0.f;
  }
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
  }
  __device__ __forceinline__ float value() const { return hi + lo; }
  // (hi + lo) - y with a single final rounding of the small part
  __device__ __forceinline__ float minus(float y) const { return (hi - y) + lo; }
  __device__ __forceinline__ double dvalue() const { return (double)hi + (double)lo; }
};
template <>
struct CSum<double> {
  double hi;
  double lo = 0.0;  // always zero: FP64 needs no compensation here
  __device__ __forceinline__ void init(double x) { hi = x; }
  __device__ __forceinline__ void add(double x) { hi += x; }
  __device__ __forceinline__ double value() const { return hi; }
  __device__ __forceinline__ double minus(double y) const { return hi - y; }
  __device__ __forceinline__ double dvalue() const { return hi; }
};

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned r;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

}  // namespace acg
