/* TEST INFRASTRUCTURE ONLY: no-op NVTX for the CPU build of the reference. */
#pragma once
static inline int nvtxRangePushA(const char*) { return 0; }
static inline int nvtxRangePop() { return 0; }
