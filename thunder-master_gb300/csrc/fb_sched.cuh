// fb_sched.cuh -- work distribution of the assembly kernels: one task per
// thread (or warp) of a grid that covers the work, or a persistent grid
// whose warps pull chunks of tasks from a device counter.  A batch of
// structures is one concatenated task list, so the persistent form balances
// uneven structures across the SMs inside one launch.
#pragma once
#include <cuda_runtime.h>
#include "fb_launch.h"

namespace fb {

// thread-per-item kernels (one lane per triplet): items are handed out in
// groups of 32 consecutive items (one per lane), q.chunk groups per grab,
// so a warp walks a contiguous run of the (binned) item order
template <class F>
__device__ __forceinline__ void for_each_item(int n, const Sched &q, F &&f) {
  if (!q.ctr) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) f(t);
    return;
  }
  int lane = threadIdx.x & 31;
  int ngroups = (n + 31) >> 5;
  for (;;) {
    int g0 = 0;
    if (lane == 0) g0 = atomicAdd(q.ctr, q.chunk);
    g0 = __shfl_sync(0xffffffffu, g0, 0);
    if (g0 >= ngroups) break;
    int g1 = min(g0 + q.chunk, ngroups);
    for (int g = g0; g < g1; g++) {
      int t = (g << 5) + lane;
      if (t < n) f(t);
    }
  }
}

// warp-per-item kernels (one warp per atom, lanes over its pairs)
template <class F>
__device__ __forceinline__ void for_each_warp_item(int n, const Sched &q, F &&f) {
  int lane = threadIdx.x & 31;
  if (!q.ctr) {
    int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w < n) f(w, lane);
    return;
  }
  for (;;) {
    int w0 = 0;
    if (lane == 0) w0 = atomicAdd(q.ctr, q.chunk);
    w0 = __shfl_sync(0xffffffffu, w0, 0);
    if (w0 >= n) break;
    int w1 = min(w0 + q.chunk, n);
    for (int w = w0; w < w1; w++) f(w, lane);
  }
}

// grid of a launch: cover the work, or a persistent grid of ctas_per_sm CTAs
// on every SM (never more CTAs than there is work for).  The counter of a
// persistent launch is cleared on the stream first.
inline int sched_launch(const KCfg &cfg, long long threads_needed, int *ctr, cudaStream_t s, dim3 &grid,
                        dim3 &block, Sched &q) {
  int bs = cfg.threads > 0 ? cfg.threads : 128;
  block = dim3(bs);
  long long cover = (threads_needed + bs - 1) / bs;
  if (cover < 1) cover = 1;
  if (cfg.ctas_per_sm > 0 && ctr) {
    long long persist = (long long)cfg.nsm * cfg.ctas_per_sm;
    grid = dim3((unsigned)(persist < cover ? persist : cover));
    q.ctr = ctr;
    q.chunk = cfg.chunk > 0 ? cfg.chunk : 1;
    cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(int), s);
    return (int)e;
  }
  grid = dim3((unsigned)cover);
  q.ctr = nullptr;
  q.chunk = 1;
  return 0;
}

}  // namespace fb
