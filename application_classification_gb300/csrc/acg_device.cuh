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
      return acg::set_error(ACG_ERR_CUDA, "%s:%d: %s: %s", __FILE__, __LINE__, \
                            #expr, cudaGetErrorString(acg_e_));               \
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

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned r;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

}  // namespace acg
