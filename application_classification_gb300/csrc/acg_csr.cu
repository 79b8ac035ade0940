// acg_csr.cu -- graph-structure primitives: exclusive scan, stable LSD radix
// sort, CSR offsets and the chunked work-item lists.
//
// The reference has no CSR: it scatters every (pattern edge, data edge) value
// with a compare-and-swap max into the endpoint's slot (ac.hxx:115-149,
// helpers.hxx:36-55).  Here both orderings of the data edges -- grouped by
// destination and grouped by source -- are built once per data graph, so every
// edge->vertex message becomes a segmented reduction with no atomics.
//
// All of this is integer, HBM-bound work; the sort is stable so that each CSR
// segment lists its edges in increasing original edge id, which makes every
// later floating-point reduction order (and so every result) deterministic.
#include <cuda_runtime.h>

#include <cstdlib>
#include <atomic>
#include <mutex>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "acg_device.cuh"
#include "acg_internal.h"

namespace acg {

// The library's memory pool on the current device (stream-ordered, never
// trimmed: freed blocks stay cached for the next data graph or plan, as a
// caching allocator does).  Created on first use per device.  ACG_MEMPOOL=0
// in the environment selects plain cudaMalloc / cudaFree instead (profilers
// that save and restore device memory between kernel replays expect it).
static cudaMemPool_t g_pools[64] = {};
static std::mutex g_pool_mutex;

// Injected allocation failure (acg_inject_alloc_failure): the value counts
// down with every device allocation of the library; the one that takes it
// from 1 to 0 fails as if the device were out of memory.
static std::atomic<long long> g_fail_nth{0};
static bool injected_failure() {
  if (g_fail_nth.load(std::memory_order_relaxed) <= 0) return false;
  return g_fail_nth.fetch_sub(1) == 1;
}
void set_alloc_failure(long long nth) { g_fail_nth.store(nth > 0 ? nth : 0); }

long long device_memory_in_use() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1;
  long long total = 0;
  uint64_t used = 0;
  {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    if (dev >= 0 && dev < 64 && g_pools[dev] &&
        cudaMemPoolGetAttribute(g_pools[dev], cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess)
      total += (long long)used;
  }
  cudaMemPool_t def = nullptr;  // the scratch of the CSR build comes from the default pool
  if (cudaDeviceGetDefaultMemPool(&def, dev) == cudaSuccess &&
      cudaMemPoolGetAttribute(def, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess)
    total += (long long)used;
  cudaGetLastError();
  return total;
}

static bool pool_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("ACG_MEMPOOL");
    return !(e && e[0] == '0');
  }();
  return on;
}

static cudaMemPool_t device_pool() {
  if (!pool_enabled()) return nullptr;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  cudaMemPool_t* pools = g_pools;
  if (!pools[dev]) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    pools[dev] = pool;
  }
  return pools[dev];
}

acg_status dev_alloc(std::vector<DevBuf>* owned, size_t bytes, void** out, cudaStream_t s) {
  if (bytes == 0) bytes = 16;
  if (injected_failure())
    return set_error(ACG_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu) failed: injected failure", bytes);
  void* p = nullptr;
  cudaMemPool_t pool = device_pool();
  cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, s) : cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(ACG_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu) failed: %s", bytes,
                     cudaGetErrorString(e));
  }
  e = cudaMemsetAsync(p, 0, bytes, s);
  if (e != cudaSuccess) {
    if (pool) {
      cudaStreamSynchronize(s);
      cudaFreeAsync(p, s);
    } else {
      cudaFree(p);
    }
    return set_error(ACG_ERR_CUDA, "cudaMemsetAsync failed: %s", cudaGetErrorString(e));
  }
  owned->push_back({p, bytes});
  *out = p;
  return ACG_OK;
}

void release_pools() {
  std::lock_guard<std::mutex> lock(g_pool_mutex);
  for (cudaMemPool_t p : g_pools)
    if (p) cudaMemPoolTrimTo(p, 0);
}

void dev_free_all(std::vector<DevBuf>* owned) {
  if (owned->empty()) return;
  // the buffers may be in use on any stream: wait for the device once, then
  // hand them back to the pool
  cudaDeviceSynchronize();
  const bool pool = pool_enabled();
  for (auto& b : *owned)
    if (b.p) {
      if (pool)
        cudaFreeAsync(b.p, 0);
      else
        cudaFree(b.p);
    }
  cudaDeviceSynchronize();
  owned->clear();
}

void dev_free_on(std::vector<DevBuf>* owned, cudaStream_t s) {
  if (owned->empty()) return;
  if (pool_enabled()) {
    for (auto& b : *owned)
      if (b.p) cudaFreeAsync(b.p, s);
  } else {
    cudaStreamSynchronize(s);
    for (auto& b : *owned)
      if (b.p) cudaFree(b.p);
  }
  owned->clear();
}

// ---------------------------------------------------------------- scan
namespace {

// Short-lived scratch of the CSR build and the work splits: the library's
// pool (which keeps its memory, so a repeated build maps nothing new), or
// plain cudaMalloc when ACG_MEMPOOL=0.
cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
  if (injected_failure()) return cudaErrorMemoryAllocation;
  cudaMemPool_t pool = device_pool();
  return pool ? cudaMallocFromPoolAsync(p, bytes, pool, s) : cudaMalloc(p, bytes);
}

void scratch_free(void* p, cudaStream_t s) {
  if (pool_enabled()) {
    cudaFreeAsync(p, s);
  } else {
    cudaStreamSynchronize(s);
    cudaFree(p);
  }
}

constexpr int kScanThreads = 1024;
constexpr int kScanPerThread = 4;
constexpr int kScanTile = kScanThreads * kScanPerThread;

// Exclusive scan of one tile per block; writes the tile total to sums[block].
template <typename T>
__global__ void __launch_bounds__(kScanThreads)
scan_tile_kernel(const T* __restrict__ in, T* __restrict__ out, size_t n, T* __restrict__ sums) {
  __shared__ T warp_tot[kScanThreads / 32];
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanPerThread;
  T v[kScanPerThread];
  T t = 0;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    v[k] = (base + k < n) ? in[base + k] : T(0);
    t += v[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  T inc = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    T w = warp_tot[lane];
    T wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_tot[lane] = wi - w;  // exclusive prefix of warp totals
    if (lane == 31 && sums) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  T run = warp_tot[warp] + inc - t;
#pragma unroll
  for (int k = 0; k < kScanPerThread; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
}

template <typename T>
__global__ void scan_add_kernel(T* __restrict__ out, size_t n, const T* __restrict__ offs) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}

template <typename T>
acg_status scan_exclusive(const T* in, T* out, size_t n, cudaStream_t s) {
  if (n == 0) return ACG_OK;
  const size_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    scan_tile_kernel<T><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
    ACG_LAUNCH_CHECK();
    return ACG_OK;
  }
  T* sums = nullptr;
  ACG_CUDA_TRY(scratch_alloc((void**)&sums, nb * sizeof(T), s));
  scan_tile_kernel<T><<<(unsigned)nb, kScanThreads, 0, s>>>(in, out, n, sums);
  ACG_LAUNCH_CHECK();
  acg_status st = scan_exclusive<T>(sums, sums, nb, s);
  if (st == ACG_OK) {
    scan_add_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums);
    if (cudaGetLastError() != cudaSuccess) st = set_error(ACG_ERR_CUDA, "scan_add launch failed");
  }
  scratch_free(sums, s);
  return st;
}

}  // namespace

acg_status scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s) {
  return scan_exclusive<uint32_t>(in, out, n, s);
}

acg_status scan_exclusive_u64(const unsigned long long* in, unsigned long long* out, size_t n,
                              cudaStream_t s) {
  return scan_exclusive<unsigned long long>(in, out, n, s);
}

// ----------------------------------------------------------- radix sort
// One warp owns one tile of kSortTile consecutive keys.  Pass structure:
// per-tile digit histograms (digit-major) -> exclusive scan -> stable scatter
// in which each warp walks its tile 32 keys at a time, ranking equal digits
// with __match_any_sync so that the original order is kept.
namespace {

constexpr int kSortTile = 4096;
constexpr int kSortWarps = 8;

__global__ void __launch_bounds__(kSortWarps * 32)
radix_hist_kernel(const uint32_t* __restrict__ keys, size_t n, int shift, int ntiles,
                  uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[kSortWarps][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * kSortWarps + w;
  for (int d = lane; d < 256; d += 32) h[w][d] = 0;
  __syncwarp();
  if (tile < ntiles) {
    const size_t lo = (size_t)tile * kSortTile;
    const size_t hi = min(n, lo + kSortTile);
    for (size_t i = lo + lane; i < hi; i += 32) atomicAdd(&h[w][(keys[i] >> shift) & 255u], 1u);
    __syncwarp();
    for (int d = lane; d < 256; d += 32) hist[(size_t)d * ntiles + tile] = h[w][d];
  }
}

__global__ void __launch_bounds__(kSortWarps * 32)
radix_scatter_kernel(const uint32_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                     uint32_t* __restrict__ kout, uint32_t* __restrict__ vout, size_t n,
                     int shift, int ntiles, const uint32_t* __restrict__ offs) {
  __shared__ uint32_t cnt[kSortWarps][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.x * kSortWarps + w;
  if (tile >= ntiles) return;  // whole warp leaves together
  for (int d = lane; d < 256; d += 32) cnt[w][d] = offs[(size_t)d * ntiles + tile];
  __syncwarp();
  const size_t lo = (size_t)tile * kSortTile;
  const size_t hi = min(n, lo + kSortTile);
  const unsigned lt = lanemask_lt();
  for (size_t b = lo; b < hi; b += 32) {
    const size_t i = b + lane;
    const bool valid = i < hi;
    const unsigned vmask = __ballot_sync(0xffffffffu, valid);
    uint32_t k = 0, v = 0, d = 0, pos = 0;
    unsigned peers = 0;
    if (valid) {
      k = kin[i];
      v = vin[i];
      d = (k >> shift) & 255u;
      peers = __match_any_sync(vmask, d);
      pos = cnt[w][d] + __popc(peers & lt);
    }
    __syncwarp();
    if (valid && (peers & lt) == 0) cnt[w][d] += __popc(peers);  // group leader
    __syncwarp();
    if (valid) {
      kout[pos] = k;
      vout[pos] = v;
    }
  }
}

}  // namespace

acg_status radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp,
                                uint32_t* vals_tmp, size_t n, int bits, cudaStream_t s) {
  if (n <= 1 || bits <= 0) return ACG_OK;
  const int ntiles = (int)((n + kSortTile - 1) / kSortTile);
  const size_t hn = (size_t)ntiles * 256;
  uint32_t* hist = nullptr;
  ACG_CUDA_TRY(scratch_alloc((void**)&hist, hn * sizeof(uint32_t), s));
  uint32_t *ka = keys, *va = vals, *kb = keys_tmp, *vb = vals_tmp;
  acg_status st = ACG_OK;
  const unsigned blocks = (unsigned)((ntiles + kSortWarps - 1) / kSortWarps);
  for (int shift = 0; shift < bits && st == ACG_OK; shift += 8) {
    radix_hist_kernel<<<blocks, kSortWarps * 32, 0, s>>>(ka, n, shift, ntiles, hist);
    if (cudaGetLastError() != cudaSuccess) {
      st = set_error(ACG_ERR_CUDA, "radix_hist launch failed");
      break;
    }
    st = scan_exclusive_u32(hist, hist, hn, s);
    if (st != ACG_OK) break;
    radix_scatter_kernel<<<blocks, kSortWarps * 32, 0, s>>>(ka, va, kb, vb, n, shift, ntiles, hist);
    if (cudaGetLastError() != cudaSuccess) {
      st = set_error(ACG_ERR_CUDA, "radix_scatter launch failed");
      break;
    }
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  if (st == ACG_OK && ka != keys) {
    cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
  }
  scratch_free(hist, s);
  return st;
}

// ------------------------------------------------------------------ CSR
namespace {

__global__ void iota_kernel(uint32_t* __restrict__ v, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

// off[v] = first position whose key >= v, for v in [0, n]; keys sorted.
__global__ void csr_offsets_kernel(const uint32_t* __restrict__ keys, int m, int n,
                                   int* __restrict__ off) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > m) return;
  const long long prev = i > 0 ? (long long)keys[i - 1] : -1;
  const long long cur = i < m ? (long long)keys[i] : (long long)n;
  for (long long v = prev + 1; v <= cur; ++v) off[v] = (int)i;
}

__global__ void gather_other_kernel(const uint32_t* __restrict__ eid,
                                    const uint32_t* __restrict__ other, int m,
                                    int* __restrict__ out) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < m) out[i] = (int)other[eid[i]];
}

}  // namespace

acg_status build_csr(const uint32_t* key, const uint32_t* other, int n, int m, Csr* out,
                     std::vector<DevBuf>* owned, cudaStream_t s) {
  out->n = n;
  out->m = m;
  ACG_TRY(dev_alloc(owned, sizeof(int) * ((size_t)n + 1), (void**)&out->off, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * (size_t)m, (void**)&out->eid, s));
  ACG_TRY(dev_alloc(owned, sizeof(int) * (size_t)m, (void**)&out->other, s));
  const size_t mm = m > 0 ? (size_t)m : 1;
  uint32_t *k = nullptr, *k2 = nullptr, *v2 = nullptr;
  {
    cudaError_t e = scratch_alloc((void**)&k, mm * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = scratch_alloc((void**)&k2, mm * sizeof(uint32_t), s);
    if (e == cudaSuccess) e = scratch_alloc((void**)&v2, mm * sizeof(uint32_t), s);
    if (e != cudaSuccess) {  // free what was taken; the CSR's own buffers are in `owned`
      cudaGetLastError();
      for (uint32_t* p : {k, k2, v2})
        if (p) scratch_free(p, s);
      return set_error(ACG_ERR_OUT_OF_MEMORY, "build_csr: scratch of %zu bytes: %s",
                       mm * sizeof(uint32_t), cudaGetErrorString(e));
    }
  }
  acg_status st = ACG_OK;
  uint32_t* vals = reinterpret_cast<uint32_t*>(out->eid);
  if (m > 0) {
    cudaMemcpyAsync(k, key, (size_t)m * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    iota_kernel<<<ceil_div(m, 256), 256, 0, s>>>(vals, (size_t)m);
    int bits = 0;
    while (bits < 32 && ((uint64_t)(n > 0 ? n - 1 : 0) >> bits) != 0) ++bits;
    st = radix_sort_pairs_u32(k, vals, k2, v2, (size_t)m, bits, s);
  }
  if (st == ACG_OK) {
    csr_offsets_kernel<<<ceil_div((long long)m + 1, 256), 256, 0, s>>>(k, m, n, out->off);
    if (m > 0) gather_other_kernel<<<ceil_div(m, 256), 256, 0, s>>>(vals, other, m, out->other);
    if (cudaGetLastError() != cudaSuccess) st = set_error(ACG_ERR_CUDA, "csr launch failed");
  }
  scratch_free(k, s);
  scratch_free(k2, s);
  scratch_free(v2, s);
  return st;
}

}  // namespace acg
