// swfd_gridsync.cuh -- a bounded grid-wide barrier for cooperative launches
// (every block of the grid resident: cudaLaunchCooperativeKernel).
#pragma once

#include "swfd_internal.h"

namespace swfd {

// the slowest wait ends after 2^24 polls whatever the timer says
constexpr long long GRID_BARRIER_MAX_POLLS = 1ll << 24;

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// after relaxed loads that observed release stores: acquire what they published
__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}
// barrier `id` (1..15) of the block's first `nthreads` threads (a multiple of 32)
__device__ __forceinline__ void bar_named(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// Wait (thread 0 of a warp group) until *flag >= v; false when the wait ran
// out (wait_ns or GRID_BARRIER_MAX_POLLS polls) or another block timed out,
// with ERR_BIT_TIMEOUT set in *err.
__device__ __forceinline__ bool wait_flag(const unsigned* flag, unsigned v, int* err,
                                          unsigned long long wait_ns) {
  const unsigned long long t0 = global_ns();
  for (long long it = 0; (int)(ld_acquire_u32(flag) - v) < 0; ++it) {
    if ((it & 63) == 63 &&
        (global_ns() - t0 > wait_ns || it > GRID_BARRIER_MAX_POLLS ||
         (*(volatile int*)err & ERR_BIT_TIMEOUT))) {
      atomicOr(err, ERR_BIT_TIMEOUT);
      return false;
    }
  }
  return true;
}

// Grid barrier number k (1, 2, ...): every block adds one to *cnt (zero at
// launch) and waits until it holds k * gridDim.x.  A block whose wait runs
// out (wait_ns, or GRID_BARRIER_MAX_POLLS polls), or that sees another
// block's timeout, sets ERR_BIT_TIMEOUT in *err and every thread of the
// block gets false; the caller then returns, so no wait outlasts its limit.
__device__ __forceinline__ bool grid_barrier(unsigned* cnt, unsigned k, int* err,
                                             unsigned long long wait_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    red_release_add_u32(cnt, 1u);
    const int good = wait_flag(cnt, k * gridDim.x, err, wait_ns) ? 1 : 0;
    __threadfence();
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

}  // namespace swfd
