// fv_tma.cuh -- TMA (cp.async.bulk.tensor) and mbarrier helpers, written as
// inline PTX (PTX ISA: "Data movement: cp.async.bulk.tensor", "Parallel
// synchronization: mbarrier").
//
// The FP64 strip kernel stages the new rows of each interior block with one
// 2-D tensor copy per field and 4-row chunk: a box of (TX + 4) x 4 doubles
// starting at column x0 - 2 (x0 a multiple of 32, so the start is 16-byte
// aligned) lands in four consecutive rows of the shared primitive ring,
// completion counted in bytes on one mbarrier per CTA.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace fv {

// TMA descriptors of the five field arrays of one state (storage order).
struct TmaState {
  CUtensorMap m[5];
};

#ifndef FV_TMA_ROWS
#define FV_TMA_ROWS 4
#endif
// rows per tensor copy (the ring's chunk): divides 4 and the tile height, and
// a chunk of (TX + 4) doubles per row is a multiple of 128 bytes (the
// alignment of a tensor copy's shared-memory destination)
constexpr int kTmaRows = FV_TMA_ROWS;

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

// Makes an initialised mbarrier visible to the async proxy.
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier shared-memory accesses (and, after a CTA
// barrier, the CTA's) before later async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            unsigned long long* m) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(m))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* m, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits for phase `parity` of m to complete, at most max_polls polls (each
// poll may suspend the thread for a while); false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(unsigned long long* m, unsigned parity, int max_polls = 1 << 22) {
  for (int i = 0; i < max_polls; ++i)
    if (mbar_try_wait(m, parity)) return true;
  return false;
}

}  // namespace fv
