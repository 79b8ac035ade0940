// acg_internal.h -- internal (non-ABI) declarations shared by the CUDA sources.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <algorithm>
#include <vector>

#include "acg.h"
#include "acg_common.h"

namespace acg {

// Device buffer owned by a data/plan object.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// A CSR ordering of the data edges.  Position i in [off[v], off[v+1]) is an
// edge whose grouping endpoint is v; positions inside a segment are in
// increasing original edge id (the sort is stable).
struct Csr {
  int n = 0;               // vertices
  int m = 0;               // edges
  int* off = nullptr;      // [n + 1]
  int* eid = nullptr;      // [m] original edge id at each position
  int* other = nullptr;    // [m] the other endpoint at each position
};

// Work of a warp-per-item segmented pass over one CSR (built on the device
// from its offsets): item = {vertex, first position, end position, partial row or
// -1}; warp w does items [wsplit[w], wsplit[w+1]), contiguous and of near-equal
// cost (load steps + a per-item overhead).  A vertex whose edges would take a
// large share of one warp's work is split into chunks that reduce into partial
// rows; heavy vertex h owns partial rows [hbase[h], hbase[h] + hcount[h]),
// combined afterwards in chunk order (no atomics: results are deterministic).
struct WarpWork {
  int4* items = nullptr;
  int nitems = 0;
  int* wsplit = nullptr;   // [nparts + 1]
  int nparts = 0;          // parts of the split: one per warp, or item ranges
  int chunk = 0;           // positions per chunk
  int* hbase = nullptr;
  int* hcount = nullptr;
  int* hvert = nullptr;
  int* pheavy = nullptr;   // [npartial] heavy vertex index of each partial row
  int nheavy = 0, npartial = 0;
};
// `step` = positions one warp loads per step of its pass (the cost unit).
// With max_ranges > 1 the work of each of the nwarps launched warps is cut into
// R = clamp(its steps / kMinRangeSteps, 1, max_ranges) item ranges (claimed at
// run time past the first); a chunk is 1 / chunk_div of a part's cost (at least
// 4 steps).
constexpr int kMinRangeSteps = 16;
// max_chunk caps the chunk length (positions) of heavy vertices.
acg_status build_warp_work(const Csr& c, int nwarps, int step, WarpWork* out,
                           std::vector<DevBuf>* owned, cudaStream_t s, int max_ranges = 1,
                           int chunk_div = 4, int max_chunk = 1 << 24);
// Parts of a split for nwarps warps whose total cost is `total` steps.
inline int work_parts(double total, int nwarps, int max_ranges) {
  if (max_ranges <= 1 || nwarps < 1) return std::max(1, nwarps);
  const double r = total / nwarps / kMinRangeSteps;
  return nwarps * (r < 1.0 ? 1 : (r > max_ranges ? max_ranges : (int)r));
}

// ---- primitives (acg_csr.cu)
// Exclusive scan of n uint32 values (in and out may alias); stream ordered.
acg_status scan_exclusive_u32(const uint32_t* in, uint32_t* out, size_t n, cudaStream_t s);
acg_status scan_exclusive_u64(const unsigned long long* in, unsigned long long* out, size_t n,
                              cudaStream_t s);
// Stable LSD radix sort of (key, value) pairs on the low `bits` key bits.
// Sorted result ends in keys/vals; keys_tmp/vals_tmp are scratch of size n.
acg_status radix_sort_pairs_u32(uint32_t* keys, uint32_t* vals, uint32_t* keys_tmp,
                                uint32_t* vals_tmp, size_t n, int bits, cudaStream_t s);
// Build the CSR grouping edges by `key[e]` (the other endpoint is `other[e]`).
acg_status build_csr(const uint32_t* key, const uint32_t* other, int n, int m, Csr* out,
                     std::vector<DevBuf>* owned, cudaStream_t s);

// Allocate `bytes` (>= 1) of device memory, zero it, record it in `owned`.
acg_status dev_alloc(std::vector<DevBuf>* owned, size_t bytes, void** out, cudaStream_t s);
void dev_free_all(std::vector<DevBuf>* owned);
// Free buffers used only on stream s, in stream order: no device-wide wait, so
// work on other streams (a feature upload) keeps running.
void dev_free_on(std::vector<DevBuf>* owned, cudaStream_t s);
// Return the pools' cached free memory to the driver (acg_release_cached_memory).
void release_pools();
// The nth device allocation from now fails (nth <= 0: none); acg_inject_alloc_failure.
void set_alloc_failure(long long nth);
// Bytes in use in the library's pool and the device's default pool (-1 on error).
long long device_memory_in_use();

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace acg
