// fv_probe.cu -- measures the FP64 FMA throughput of the current GPU, and
// exercises the bounded waits: the mbarrier wait of the TMA staging path and
// the grid barrier of the multi-step kernel.
//
// The bit-exact FP64 stage kernels are bound by the FP64 pipe, not by HBM,
// so their roofline is the FP64 instruction rate.  fvgpu_probe_fp64_rate
// measures it with a throughput loop: every thread of a full-occupancy grid
// runs eight independent fma chains (enough independent work to cover the
// pipe latency), timed with CUDA events after one warm-up launch.
#include <cuda_runtime.h>

#include "fv3d_gb300.h"
#include "fv_grid.cuh"
#include "fv_tma.cuh"

namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) dfma_loop(double a, double b, int iters, double* sink) {
  double x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (double)(threadIdx.x + c) * 1.0e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == -1.0) sink[0] = s;  // keeps the chains live; never true for these inputs
}

// One CTA waits on a fresh mbarrier with the stage kernels' bounded wait;
// thread 0 arrives on it first only when `arrive` is set.  out[0] = 1 when
// the wait completed, 0 when it gave up.
__global__ void __launch_bounds__(kThreads) wait_probe(int arrive, int max_polls, int* out) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    fv::mbar_init(&bar, 1);
    fv::fence_mbar_init();
  }
  __syncthreads();
  if (arrive && threadIdx.x == 0) fv::mbar_arrive_expect_tx(&bar, 0);
  const bool ok = fv::mbar_wait(&bar, 0, max_polls);
  __syncthreads();
  if (threadIdx.x == 0) out[0] = ok ? 1 : 0;
}

// Two resident CTAs meet at the multi-step kernel's grid barrier; CTA 1
// arrives only when `arrive_all` is set.  out[0] = 1 when CTA 0's wait
// completed, 0 when it gave up.
__global__ void __launch_bounds__(kThreads) grid_wait_probe(fv::GridBarrier gb, int arrive_all, int max_polls,
                                                            int* out) {
  if (blockIdx.x == 1 && !arrive_all) return;  // never arrives
  const bool ok = fv::grid_sync(gb, 0, max_polls);
  if (blockIdx.x == 0 && threadIdx.x == 0) out[0] = ok ? 1 : 0;
}

}  // namespace

extern "C" int fvgpu_probe_grid_wait(int arrive_all, int max_polls) {
  if (max_polls < 1) return FV_ERR_PARAM;
  unsigned* d = nullptr;  // barrier counter, abort flag, result
  int h = -1;
  if (cudaMalloc(&d, 3 * sizeof(unsigned)) != cudaSuccess) return FV_ERR_NOMEM;
  bool ok = cudaMemset(d, 0, 3 * sizeof(unsigned)) == cudaSuccess;
  if (ok) {
    const fv::GridBarrier gb{d, reinterpret_cast<int*>(d + 1)};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2);
    cfg.blockDim = dim3(kThreads);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    ok = cudaLaunchKernelEx(&cfg, grid_wait_probe, gb, arrive_all ? 1 : 0, max_polls,
                            reinterpret_cast<int*>(d + 2)) == cudaSuccess &&
         cudaMemcpy(&h, d + 2, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(d);
  if (!ok) return FV_ERR_CUDA;
  return h == 1 ? FV_OK : FV_ERR_TIMEOUT;
}

extern "C" int fvgpu_probe_wait(int arrive, int max_polls) {
  if (max_polls < 1) return FV_ERR_PARAM;
  int* d = nullptr;
  int h = -1;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return FV_ERR_NOMEM;
  wait_probe<<<1, kThreads>>>(arrive ? 1 : 0, max_polls, d);
  const bool ok = cudaGetLastError() == cudaSuccess && cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  cudaFree(d);
  if (!ok) return FV_ERR_CUDA;
  return h == 1 ? FV_OK : FV_ERR_TIMEOUT;
}

extern "C" int fvgpu_probe_fp64_rate(double* lane_ops_per_s) {
  if (!lane_ops_per_s) return FV_ERR_PARAM;
  *lane_ops_per_s = 0.0;
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dfma_loop, kThreads, 0) != cudaSuccess)
    return FV_ERR_CUDA;
  double* sink = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess) return FV_ERR_NOMEM;
  int rc = FV_OK;
  const int blocks = sms * (per_sm > 0 ? per_sm : 1);
  const int iters = 4096;
  float ms = 0.f;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = FV_ERR_CUDA;
  } else {
    dfma_loop<<<blocks, kThreads>>>(0.999999, 1.0e-7, iters, sink);  // warm-up
    cudaEventRecord(e0);
    dfma_loop<<<blocks, kThreads>>>(0.999999, 1.0e-7, iters, sink);
    cudaEventRecord(e1);
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || ms <= 0.f)
      rc = FV_ERR_CUDA;
  }
  if (rc == FV_OK)
    *lane_ops_per_s = (double)blocks * kThreads * (double)iters * kChains / (ms * 1.0e-3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(sink);
  return rc;
}
