// fv_grid.cuh -- a grid-wide barrier with a bounded wait, for kernels
// launched cooperatively (every CTA resident at once).
//
// Each CTA arrives on a counter in global memory (release: a GPU-scope fence
// before the arrival) and one thread polls it with acquire loads until the
// whole grid has arrived.  The wait is bounded: after max_polls polls (about
// a second with the sleep between polls) the CTA raises a shared abort flag,
// reports failure and its kernel returns; a CTA that sees the abort flag
// gives up as well, so one missing CTA ends every wait instead of hanging the
// GPU.  The counter counts arrivals over the whole launch: barrier number k
// (from 0) completes at (k + 1) * gridDim.x arrivals; the host zeroes the
// counter and the flag before each launch.
#pragma once

namespace fv {

constexpr int kGridBarrierPolls = 1 << 24;

struct GridBarrier {
  unsigned* count;  // arrivals so far
  int* abort;       // set when any CTA gave up waiting
};

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Barrier number k of the launch.  Every thread of every CTA calls it; false
// when the wait ran out (or another CTA's did): the caller returns.
__device__ __forceinline__ bool grid_sync(const GridBarrier& gb, unsigned k, int max_polls = kGridBarrierPolls) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(gb.count, 1u);
    const unsigned target = (k + 1u) * gridDim.x;
    int ok = 1, polls = 0;
    while (ld_acquire_gpu(gb.count) < target) {
      if (*(volatile int*)gb.abort != 0 || ++polls > max_polls) {
        ok = 0;
        atomicExch(gb.abort, 1);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace fv
