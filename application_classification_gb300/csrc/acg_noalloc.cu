// acg_noalloc.cu -- acg_initial_mu_noalloc: the match's initial mu without any
// memory allocation.
//
// Who needs it: callers that cannot allocate device memory at the point of the
// call -- code running while a CUDA stream is being captured into a graph
// (where cudaMalloc is not allowed), serving loops that run under a fixed,
// pre-reserved memory budget, and hosts that embed this library inside another
// framework whose allocator they must not bypass.  They can still pass their own
// input and output buffers; what they cannot provide is the kernel's scratch.
//
// So the scratch of this entry point -- the per-block log-sum-exp partials of
// the column normaliser and the finished normaliser -- lives in one file-scope
// device array of fixed size (188,544 doubles, about 1.5 MB), which every
// GPU that loads the library holds until the process exits.  Host code cannot
// use the array's name as a device address (in host code it names a host-side
// stand-in), so the address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on it.
// That first call therefore does a runtime query: make it before any stream
// capture begins.  The address is kept per device together with the identity
// of the CUDA context it was looked up in; after cudaDeviceReset (which
// unloads the module and the array with it) the device's next context has
// another identity, so the next call looks the address up again -- that call,
// too, must come before any capture.  Every call uses the same array: calls
// whose kernels overlap on the GPU (two streams, two threads) race on it and
// must be serialised by the caller.  Nothing in the array needs to start at
// zero: each call writes every partial it later reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "acg.h"
#include "acg_common.h"
#include "acg_device.cuh"

namespace {

constexpr int kNaThreads = 256;
constexpr int kNaMaxCols = 128;    // pattern vertices
constexpr int kNaMaxDim = 32;      // feature dimension
constexpr int kNaMaxBlocks = 736;  // blocks of the statistics pass
constexpr int kScratchDoubles = kNaMaxBlocks * kNaMaxCols * 2 + kNaMaxCols;  // 188,544 doubles

// partials [block][column] as (max, scaled sum), then the column LSE
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
double* g_scratch_ptr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};  // context the address belongs to

// Unique id of the current CUDA context (0 if none or unknown), from the
// driver's cuCtxGetCurrent / cuCtxGetId, found through the runtime's entry
// point query so that no driver library is linked.  A host-side query: it
// enqueues nothing and is allowed while a stream is captured.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetId>(f);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Distance in the difference form, summed over the feature index in order
// (ac.hxx:33-56), the same arithmetic as the main cdist kernel's FP64 path.
__device__ __forceinline__ double dist_row(const double* __restrict__ x, const double* y, int K) {
  double acc = 0.0;
  for (int k = 0; k < K; ++k) {
    const double d = y[k] - __ldg(x + k);
    acc += d * d;
  }
  return sqrt(acc);
}

// Pass 1: per column p, log-sum-exp over rows of -dist; one partial per block.
__global__ void __launch_bounds__(kNaThreads)
prior_stats_kernel(const double* __restrict__ x, long long n, int K, const double* __restrict__ y,
                   int P, double* __restrict__ scratch) {
  __shared__ double s_y[kNaMaxCols * kNaMaxDim];
  __shared__ double s_m[kNaThreads], s_s[kNaThreads];
  for (int t = threadIdx.x; t < P * K; t += kNaThreads) s_y[t] = y[t];
  __syncthreads();
  const int R = kNaThreads / P;  // rows per block step
  const int p = threadIdx.x % P, rl = threadIdx.x / P;
  acg::OnlineLse<double> l;
  l.init();
  if (rl < R)
    for (long long r = (long long)blockIdx.x * R + rl; r < n; r += (long long)gridDim.x * R)
      l.add(-dist_row(x + (size_t)r * K, s_y + p * K, K));
  s_m[threadIdx.x] = l.m;
  s_s[threadIdx.x] = l.s;
  __syncthreads();
  for (int c = threadIdx.x; c < P; c += kNaThreads) {
    double m = -CUDART_INF, s = 0.0;
    for (int rr = 0; rr < R; ++rr) acg::lse_merge(m, s, s_m[rr * P + c], s_s[rr * P + c]);
    scratch[((size_t)blockIdx.x * P + c) * 2] = m;
    scratch[((size_t)blockIdx.x * P + c) * 2 + 1] = s;
  }
}

// Pass 2: combine the block partials of every column in block order.
__global__ void prior_finalize_kernel(double* __restrict__ scratch, int nblocks, int P) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= P) return;
  acg::LseD l;
  l.init();
  for (int b = 0; b < nblocks; ++b) l.merge(scratch[((size_t)b * P + c) * 2], scratch[((size_t)b * P + c) * 2 + 1]);
  scratch[(size_t)kNaMaxBlocks * kNaMaxCols * 2 + c] = l.value();
}

// Pass 3: mu[r][p] = -dist(r, p) - LSE_p.
__global__ void __launch_bounds__(kNaThreads)
prior_output_kernel(const double* __restrict__ x, long long n, int K, const double* __restrict__ y,
                    int P, const double* __restrict__ scratch, double* __restrict__ mu) {
  __shared__ double s_y[kNaMaxCols * kNaMaxDim];
  for (int t = threadIdx.x; t < P * K; t += kNaThreads) s_y[t] = y[t];
  __syncthreads();
  const double* lse = scratch + (size_t)kNaMaxBlocks * kNaMaxCols * 2;
  const long long total = n * P;
  for (long long i = (long long)blockIdx.x * kNaThreads + threadIdx.x; i < total;
       i += (long long)gridDim.x * kNaThreads) {
    const long long r = i / P;
    const int p = (int)(i % P);
    mu[i] = -dist_row(x + (size_t)r * K, s_y + p * K, K) - lse[p];
  }
}

}  // namespace

extern "C" acg_status acg_initial_mu_noalloc(const double* data_node_feats, uint64_t num_nodes,
                                             uint64_t feat_dim, const double* pattern_node_feats,
                                             uint64_t pattern_nodes, double* mu_out, void* stream) {
  acg::clear_error();
  // an error left by earlier work on this thread is reported as such, not as
  // a failure of this call's launches
  if (const cudaError_t pend = cudaGetLastError(); pend != cudaSuccess)
    return acg::set_error(ACG_ERR_CUDA,
                          "acg_initial_mu_noalloc: a CUDA error from before this call was pending: %s",
                          cudaGetErrorString(pend));
  if (pattern_nodes == 0 || pattern_nodes > (uint64_t)kNaMaxCols)
    return acg::set_error(ACG_ERR_UNSUPPORTED,
                          "acg_initial_mu_noalloc: %llu pattern vertices; it supports 1..%d",
                          (unsigned long long)pattern_nodes, kNaMaxCols);
  if (feat_dim == 0 || feat_dim > (uint64_t)kNaMaxDim)
    return acg::set_error(ACG_ERR_UNSUPPORTED,
                          "acg_initial_mu_noalloc: feature dimension %llu; it supports 1..%d",
                          (unsigned long long)feat_dim, kNaMaxDim);
  if (num_nodes > (1ull << 40))
    return acg::set_error(ACG_ERR_UNSUPPORTED, "acg_initial_mu_noalloc: %llu data vertices",
                          (unsigned long long)num_nodes);
  if (num_nodes == 0) return ACG_OK;
  if (!data_node_feats || !pattern_node_feats || !mu_out)
    return acg::set_error(ACG_ERR_INVALID_ARGUMENT, "acg_initial_mu_noalloc: null pointer");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return acg::set_error(ACG_ERR_CUDA, "acg_initial_mu_noalloc: cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return acg::set_error(ACG_ERR_UNSUPPORTED, "acg_initial_mu_noalloc: device %d", dev);
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mu);
    const unsigned long long ctx = current_context_id();
    // once per device and context, with that device current
    if (!g_scratch_ptr[dev] || (ctx != 0 && ctx != g_scratch_ctx[dev])) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return acg::set_error(ACG_ERR_CUDA, "acg_initial_mu_noalloc: cudaGetSymbolAddress: %s",
                              cudaGetErrorString(e));
      g_scratch_ptr[dev] = static_cast<double*>(p);
      g_scratch_ctx[dev] = ctx ? ctx : current_context_id();
    }
    scratch = g_scratch_ptr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int P = (int)pattern_nodes, K = (int)feat_dim;
  const long long n = (long long)num_nodes;
  const int R = kNaThreads / P;
  const int nb = (int)std::min<long long>(kNaMaxBlocks, (n + R - 1) / R);
  prior_stats_kernel<<<nb, kNaThreads, 0, s>>>(data_node_feats, n, K, pattern_node_feats, P, scratch);
  prior_finalize_kernel<<<1, kNaMaxCols, 0, s>>>(scratch, nb, P);
  const long long total = n * P;
  const int ob = (int)std::min<long long>(kNaMaxBlocks, (total + kNaThreads - 1) / kNaThreads);
  prior_output_kernel<<<ob, kNaThreads, 0, s>>>(data_node_feats, n, K, pattern_node_feats, P,
                                                scratch, mu_out);
  e = cudaGetLastError();
  if (e != cudaSuccess)
    return acg::set_error(ACG_ERR_CUDA, "acg_initial_mu_noalloc: launch: %s", cudaGetErrorString(e));
  return ACG_OK;
}
