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

// A reduction word (the persistent 1D solve): the bits of the block's maximum
// of values >= 0 (findalpha terms; the bit patterns order as the values do
// and the sign bit is free) with the sign bit set when one of its cells
// failed checkpositivity.  GRID_WORD_EMPTY (all ones, a negative NaN) is
// never a word.
constexpr unsigned long long GRID_WORD_BAD = 1ull << 63;
constexpr unsigned long long GRID_WORD_EMPTY = ~0ull;

__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}

// Grid reduction k (1, 2, ...) on the block's first two warps (named
// barrier 1), over `red` (three sets of gridDim.x words, SWFD_SOLVE1D_WSTRIDE
// apart, filled with ones before the launch): the maximum
// alpha bits `ab` and flag `f` of the lanes fold into the block's word,
// which thread 0 posts in set k % 3 (a relaxed store; the caller's thread 0
// issued a gpu-scope fence after its last store -- the emptying of its word
// at reduction k - 1 -- while warp 1 computed findalpha, so fence and store
// form a release); then the 64 threads poll the
// grid's words of set k % 3 until none is empty, and *am, *bad (shared)
// receive the grid's maximum and flag.  The words are the only values read
// from other blocks, so the polls need no acquire fence (a gpu-scope fence
// here measured ~3 us).  Thread 0 then empties its word of set (k + 2) % 3
// for reduction k + 2: every block has posted reduction k, after reading
// every word of reduction k - 1 (set (k + 2) % 3), and the emptying store
// follows the polls that saw those posts; a block polls that set again only
// after it has seen this block's word of reduction k + 1, released after
// the emptying.  Returns false when the wait ran out (ERR_BIT_TIMEOUT in
// *err: after wait_ns, GRID_BARRIER_MAX_POLLS rounds, or another block's
// timeout).
__device__ __forceinline__ bool grid_reduce_2w(unsigned long long* red, unsigned k, int* err,
                                               unsigned long long wait_ns, unsigned long long ab,
                                               int f, double* am, int* bad) {
  __shared__ unsigned long long wv[2];
  __shared__ int wf[2], wok[2];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int G = gridDim.x;
  for (int o = 16; o > 0; o >>= 1) ab = umax64(ab, __shfl_xor_sync(0xffffffffu, ab, o));
  f = __any_sync(0xffffffffu, f);
  if (lane == 0) wv[w] = ab, wf[w] = f;
  bar_named(1, 64);
  // word j of set k % 3 at set + j * W, a 128-byte line of its own: the
  // grid's polls of one word go to one line, not the whole set's to a few
  constexpr int W = SWFD_SOLVE1D_WSTRIDE;
  unsigned long long* set = red + (size_t)(k % 3) * G * W;
  if (tid == 0)
    st_relaxed_u64(set + (size_t)blockIdx.x * W,
                   umax64(wv[0], wv[1]) | ((wf[0] | wf[1]) ? GRID_WORD_BAD : 0ull));
  // thread tid polls words tid, tid + 64, ... (at most SWFD_SOLVE1D_POLL),
  // all of them in each round
  unsigned long long m = 0;
  int fl = 0, pend = 0, ok = 1;
#pragma unroll
  for (int s = 0; s < SWFD_SOLVE1D_POLL; ++s)
    if (tid + 64 * s < G) pend |= 1 << s;
  const unsigned long long t0 = global_ns();
  for (long long it = 0; pend; ++it) {
    unsigned long long v[SWFD_SOLVE1D_POLL];
#pragma unroll
    for (int s = 0; s < SWFD_SOLVE1D_POLL; ++s)
      v[s] = (pend >> s) & 1 ? ld_relaxed_u64(set + (size_t)(tid + 64 * s) * W) : GRID_WORD_EMPTY;
#pragma unroll
    for (int s = 0; s < SWFD_SOLVE1D_POLL; ++s)
      if (v[s] != GRID_WORD_EMPTY) {
        m = umax64(m, v[s] & ~GRID_WORD_BAD);
        fl |= (int)(v[s] >> 63);
        pend &= ~(1 << s);
      }
    if (pend && (it & 63) == 63 &&
        (global_ns() - t0 > wait_ns || it > GRID_BARRIER_MAX_POLLS ||
         (*(volatile int*)err & ERR_BIT_TIMEOUT))) {
      atomicOr(err, ERR_BIT_TIMEOUT);
      ok = 0;
      break;
    }
  }
  for (int o = 16; o > 0; o >>= 1) m = umax64(m, __shfl_xor_sync(0xffffffffu, m, o));
  fl = __any_sync(0xffffffffu, fl);
  ok = __all_sync(0xffffffffu, ok);
  bar_named(1, 64);  // thread 0 has read wv, wf
  if (lane == 0) wv[w] = m, wf[w] = fl, wok[w] = ok;
  bar_named(1, 64);
  const bool good = wok[0] && wok[1];
  if (tid == 0) {
    *am = __longlong_as_double((long long)umax64(wv[0], wv[1]));
    *bad = wf[0] | wf[1];
    if (good)
      st_relaxed_u64(red + ((size_t)((k + 2) % 3) * G + blockIdx.x) * W, GRID_WORD_EMPTY);
  }
  return good;
}

}  // namespace swfd
